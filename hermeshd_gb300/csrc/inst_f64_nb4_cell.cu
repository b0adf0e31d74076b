// Stage kernels except the face kernel: T = double, nbasis 4, iquad 2.
#include "dg_launch.cuh"

namespace hermes {
KernelSet kernels_f64_nb4() {
    KernelSet k = Launch<double, 4, 2>::set();
    k.face = &face_f64_nb4;
    return k;
}
}  // namespace hermes

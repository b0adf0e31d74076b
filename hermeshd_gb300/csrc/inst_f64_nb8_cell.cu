// Stage kernels except the face kernel: T = double, nbasis 8, iquad 2.
#include "dg_launch.cuh"

namespace hermes {
KernelSet kernels_f64_nb8() {
    KernelSet k = Launch<double, 8, 2>::set();
    k.face = &face_f64_nb8;
    return k;
}
}  // namespace hermes

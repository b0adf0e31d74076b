// Stage kernels except the face kernel: T = double, nbasis 10, iquad 3.
#include "dg_launch.cuh"

namespace hermes {
KernelSet kernels_f64_nb10() {
    KernelSet k = Launch<double, 10, 3>::set();
    k.face = &face_f64_nb10;
    return k;
}
}  // namespace hermes

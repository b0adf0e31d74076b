// Stage kernels except the face kernel: T = float, nbasis 10, iquad 3.
#include "dg_launch.cuh"

namespace hermes {
KernelSet kernels_f32_nb10() {
    KernelSet k = Launch<float, 10, 3>::set();
    k.face = &face_f32_nb10;
    return k;
}
}  // namespace hermes

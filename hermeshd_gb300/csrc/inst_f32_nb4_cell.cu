// Stage kernels except the face kernel: T = float, nbasis 4, iquad 2.
#include "dg_launch.cuh"

namespace hermes {
KernelSet kernels_f32_nb4() {
    KernelSet k = Launch<float, 4, 2>::set();
    k.face = &face_f32_nb4;
    return k;
}
}  // namespace hermes

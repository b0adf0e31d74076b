// Stage kernels except the face kernel: T = float, nbasis 8, iquad 2.
#include "dg_launch.cuh"

namespace hermes {
KernelSet kernels_f32_nb8() {
    KernelSet k = Launch<float, 8, 2>::set();
    k.face = &face_f32_nb8;
    return k;
}
}  // namespace hermes

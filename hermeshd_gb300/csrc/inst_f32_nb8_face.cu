// Face kernel launcher: T = float, nbasis 8, iquad 2.
#include "dg_launch.cuh"

namespace hermes {
void face_f32_nb8(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s) {
    Launch<float, 8, 2>::face(dir, Q, flux, a, s);
}
}  // namespace hermes

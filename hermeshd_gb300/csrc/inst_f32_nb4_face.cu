// Face kernel launcher: T = float, nbasis 4, iquad 2.
#include "dg_launch.cuh"

namespace hermes {
void face_f32_nb4(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s) {
    Launch<float, 4, 2>::face(dir, Q, flux, a, s);
}
}  // namespace hermes

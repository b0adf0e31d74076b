// Face kernel launcher: T = float, nbasis 10, iquad 3.
#include "dg_launch.cuh"

namespace hermes {
void face_f32_nb10(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s) {
    Launch<float, 10, 3>::face(dir, Q, flux, a, s);
}
}  // namespace hermes

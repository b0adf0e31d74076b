// Face kernel launcher: T = double, nbasis 4, iquad 2.
#include "dg_launch.cuh"

namespace hermes {
void face_f64_nb4(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s) {
    Launch<double, 4, 2>::face(dir, Q, flux, a, s);
}
}  // namespace hermes

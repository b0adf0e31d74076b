// Generated launcher translation unit (one of four per instantiation, compiled in parallel).
#include "dg_launch.cuh"

namespace hermes {
// T = float, nbasis 8, iquad 2: face kernels with the stochastic stress
void facen_f32_nb8(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s) { Launch<float, 8, 2>::face<true>(dir, Q, flux, a, s); }
}  // namespace hermes

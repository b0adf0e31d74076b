// Generated launcher translation unit (one of four per instantiation, compiled in parallel).
#include "dg_launch.cuh"

namespace hermes {
// T = float, nbasis 10, iquad 3: face kernels with the stochastic stress
void facen_f32_nb10(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s) { Launch<float, 10, 3>::face<true>(dir, Q, flux, a, s); }
}  // namespace hermes

// Generated launcher translation unit (one of four per instantiation, compiled in parallel).
#include "dg_launch.cuh"

namespace hermes {
// T = double, nbasis 4, iquad 2: face kernels with the stochastic stress
void facen_f64_nb4(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s) { Launch<double, 4, 2>::face<true>(dir, Q, flux, a, s); }
}  // namespace hermes

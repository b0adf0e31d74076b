// Generated launcher translation unit (one of four per instantiation, compiled in parallel).
#include "dg_launch.cuh"

namespace hermes {
// T = double, nbasis 8, iquad 2: cell kernel with the stochastic stress
void celln_f64_nb8(const void* Qin, const void* Q0, void* out, const void* flux, const CellArgs& a, cudaStream_t s) {
    Launch<double, 8, 2>::cell<true>(Qin, Q0, out, flux, a, s);
}
cudaError_t prepn_f64_nb8() { return Launch<double, 8, 2>::prepare_cell<true>(); }
}  // namespace hermes

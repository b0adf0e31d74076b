// Generated launcher translation unit (one of four per instantiation, compiled in parallel).
#include "dg_launch.cuh"

namespace hermes {
// T = float, nbasis 10, iquad 3: cell kernel with the stochastic stress
void celln_f32_nb10(const void* Qin, const void* Q0, void* out, const void* flux, const CellArgs& a, cudaStream_t s) {
    Launch<float, 10, 3>::cell<true>(Qin, Q0, out, flux, a, s);
}
cudaError_t prepn_f32_nb10() { return Launch<float, 10, 3>::prepare_cell<true>(); }
}  // namespace hermes

// Generated launcher translation unit (one of four per instantiation, compiled in parallel).
#include "dg_launch.cuh"

namespace hermes {
// T = float, nbasis 4, iquad 2: cell kernel with the stochastic stress
void celln_f32_nb4(const void* Qin, const void* Q0, void* out, const void* flux, const CellArgs& a, cudaStream_t s) {
    Launch<float, 4, 2>::cell<true>(Qin, Q0, out, flux, a, s);
}
cudaError_t prepn_f32_nb4() { return Launch<float, 4, 2>::prepare_cell<true>(); }
}  // namespace hermes

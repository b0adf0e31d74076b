// Generated launcher translation unit (one of four per instantiation, compiled in parallel).
#include "dg_launch.cuh"

namespace hermes {
// T = float, nbasis 8, iquad 2: cell kernel without noise
void cell_f32_nb8(const void* Qin, const void* Q0, void* out, const void* flux, const CellArgs& a, cudaStream_t s) {
    Launch<float, 8, 2>::cell<false>(Qin, Q0, out, flux, a, s);
}
cudaError_t prep_f32_nb8() { return Launch<float, 8, 2>::prepare_cell<false>(); }
}  // namespace hermes

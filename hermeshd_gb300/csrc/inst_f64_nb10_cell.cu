// Generated launcher translation unit (one of four per instantiation, compiled in parallel).
#include "dg_launch.cuh"

namespace hermes {
// T = double, nbasis 10, iquad 3: cell kernel without noise
void cell_f64_nb10(const void* Qin, const void* Q0, void* out, const void* flux, const CellArgs& a, cudaStream_t s) {
    Launch<double, 10, 3>::cell<false>(Qin, Q0, out, flux, a, s);
}
cudaError_t prep_f64_nb10() { return Launch<double, 10, 3>::prepare_cell<false>(); }
}  // namespace hermes

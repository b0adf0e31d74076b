// Adjoint translation unit: the cell pass with one dual-number pass per column
// (ivis 2, the Tait equation of state), FP64, nbasis 10, iquad 3.
#include "dg_adjoint.cuh"

namespace hermes {
cudaError_t cell_adj_gen_nb10(const double* Q, const double* mu, const double* tadj, double* out, const AdjArgs& a,
                               cudaStream_t s) {
    return cell_adj_launch<10, 3, ADJ_GEN>(Q, mu, tadj, out, a, s);
}
}  // namespace hermes

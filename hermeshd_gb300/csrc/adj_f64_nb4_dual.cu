// Adjoint translation unit: the dual-number cell pass (the check path of the
// reverse sweep), FP64, nbasis 4, iquad 2.
#include "dg_adjoint.cuh"

namespace hermes {
cudaError_t cell_adj_dual_nb4(const double* Q, const double* mu, const double* tadj, double* out, const AdjArgs& a,
                               cudaStream_t s) {
    return cell_adj_launch<4, 2, ADJ_DUAL>(Q, mu, tadj, out, a, s);
}
}  // namespace hermes

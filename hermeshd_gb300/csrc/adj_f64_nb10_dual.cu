// Adjoint translation unit: the dual-number cell pass (the check path of the
// reverse sweep), FP64, nbasis 10, iquad 3.
#include "dg_adjoint.cuh"

namespace hermes {
cudaError_t cell_adj_dual_nb10(const double* Q, const double* mu, const double* tadj, double* out, const AdjArgs& a,
                               cudaStream_t s) {
    return cell_adj_launch<10, 3, ADJ_DUAL>(Q, mu, tadj, out, a, s);
}
}  // namespace hermes

// Adjoint translation unit: the reverse-sweep cell pass, FP64, nbasis 4, iquad 2.
#include "dg_adjoint.cuh"

namespace hermes {
cudaError_t cell_adj_rev_nb4(const double* Q, const double* mu, const double* tadj, double* out, const AdjArgs& a,
                              cudaStream_t s) {
    return cell_adj_launch<4, 2, ADJ_REV>(Q, mu, tadj, out, a, s);
}
}  // namespace hermes

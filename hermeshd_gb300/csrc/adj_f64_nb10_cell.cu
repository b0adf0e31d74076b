// Adjoint translation unit: the reverse-sweep cell pass, FP64, nbasis 10, iquad 3.
#include "dg_adjoint.cuh"

namespace hermes {
cudaError_t cell_adj_rev_nb10(const double* Q, const double* mu, const double* tadj, double* out, const AdjArgs& a,
                              cudaStream_t s) {
    return cell_adj_launch<10, 3, ADJ_REV>(Q, mu, tadj, out, a, s);
}
}  // namespace hermes

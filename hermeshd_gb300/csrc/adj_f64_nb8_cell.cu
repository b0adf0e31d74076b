// Adjoint translation unit: the reverse-sweep cell pass, FP64, nbasis 8, iquad 2.
#include "dg_adjoint.cuh"

namespace hermes {
cudaError_t cell_adj_rev_nb8(const double* Q, const double* mu, const double* tadj, double* out, const AdjArgs& a,
                              cudaStream_t s) {
    return cell_adj_launch<8, 2, ADJ_REV>(Q, mu, tadj, out, a, s);
}
}  // namespace hermes

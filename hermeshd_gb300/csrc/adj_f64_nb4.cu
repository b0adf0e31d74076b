// Adjoint launcher translation unit: FP64, nbasis 4, iquad 2.
#include "dg_adjoint.cuh"

namespace hermes {
cudaError_t adj_f64_nb4(const double* Q, const double* mu, double* tadj, double* out, const AdjArgs& a, cudaStream_t s) {
    return adj_launch<4, 2>(Q, mu, tadj, out, a, s);
}
cudaError_t limit_adj_f64_nb4(const double* Q, const double* lam_out, double* lam_in, const Geom& G, const Phys& ph,
                               cudaStream_t s) {
    return limit_adj_launch<4, 2>(Q, lam_out, lam_in, G, ph, s);
}
}  // namespace hermes

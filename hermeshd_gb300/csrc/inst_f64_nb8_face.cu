// Generated launcher translation unit (one of four per instantiation, compiled in parallel).
#include "dg_launch.cuh"

namespace hermes {
// T = double, nbasis 8, iquad 2: face kernels without noise, limiter, CFL reduction, face traces
void face_f64_nb8(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s) { Launch<double, 8, 2>::face<false>(dir, Q, flux, a, s); }
void limit_f64_nb8(void* Q, const Geom& G, const Phys& ph, cudaStream_t s) { Launch<double, 8, 2>::limit(Q, G, ph, s); }
void mindt_f64_nb8(const void* Q, const DtArgs& a, cudaStream_t s) { Launch<double, 8, 2>::mindt(Q, a, s); }
void trace_f64_nb8(const void* Q, void* tr, const Geom& G, cudaStream_t s, int v0, int nv) {
    Launch<double, 8, 2>::trace(Q, tr, G, s, v0, nv);
}
}  // namespace hermes

// Generated launcher translation unit (one of four per instantiation, compiled in parallel).
#include "dg_launch.cuh"

namespace hermes {
// T = float, nbasis 4, iquad 2: face kernels without noise, limiter, CFL reduction
void face_f32_nb4(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s) { Launch<float, 4, 2>::face<false>(dir, Q, flux, a, s); }
void limit_f32_nb4(void* Q, const Geom& G, const Phys& ph, cudaStream_t s) { Launch<float, 4, 2>::limit(Q, G, ph, s); }
void mindt_f32_nb4(const void* Q, const DtArgs& a, cudaStream_t s) { Launch<float, 4, 2>::mindt(Q, a, s); }
}  // namespace hermes

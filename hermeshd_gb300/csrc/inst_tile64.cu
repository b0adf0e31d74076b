// Launcher translation unit of the fused stage (dg_tile.cuh) of the linear
// basis in FP64, with and without the stochastic stress (inst_tile.cu: FP32).
#include "dg_launch.cuh"

namespace hermes {
void tile_f64_nb4(const void* a, const void* b, void* c, unsigned n, const TileArgs& t, cudaStream_t s) { TileLaunch<double, false>::tile(a, b, c, n, t, s); }
void tilen_f64_nb4(const void* a, const void* b, void* c, unsigned n, const TileArgs& t, cudaStream_t s) { TileLaunch<double, true>::tile(a, b, c, n, t, s); }
void dtlim_f64_nb4(void* q, const DtArgs& a, cudaStream_t s) { TileLaunch<double, false>::mindt_limit(q, a, s); }
cudaError_t tprep_f64_nb4() { return TileLaunch<double, false>::prepare(); }
cudaError_t tprepn_f64_nb4() { return TileLaunch<double, true>::prepare(); }
}  // namespace hermes

// Launcher translation unit of the fused stage (dg_tile.cuh) of the linear
// basis in FP32, with and without the stochastic stress (inst_tile64.cu: FP64).
#include "dg_launch.cuh"

namespace hermes {
void tile_f32_nb4(const void* a, const void* b, void* c, unsigned n, const TileArgs& t, cudaStream_t s) { TileLaunch<float, false>::tile(a, b, c, n, t, s); }
void tilen_f32_nb4(const void* a, const void* b, void* c, unsigned n, const TileArgs& t, cudaStream_t s) { TileLaunch<float, true>::tile(a, b, c, n, t, s); }
void dtlim_f32_nb4(void* q, const DtArgs& a, cudaStream_t s) { TileLaunch<float, false>::mindt_limit(q, a, s); }
cudaError_t tprep_f32_nb4() { return TileLaunch<float, false>::prepare(); }
cudaError_t tprepn_f32_nb4() { return TileLaunch<float, true>::prepare(); }
}  // namespace hermes

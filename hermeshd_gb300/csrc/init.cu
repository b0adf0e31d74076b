// Launcher of the initial-state kernel (dg_init.cuh).
#include "dg_init.cuh"

namespace hermes {
cudaError_t init_launch(int precision, void* Q, const InitArgs& a, cudaStream_t s) {
    if (a.ncell <= 0) return cudaSuccess;
    const unsigned nblk = (unsigned)((a.ncell + INIT_TPB - 1) / INIT_TPB);
    if (precision == 64) k_init<double><<<nblk, INIT_TPB, 0, s>>>(static_cast<double*>(Q), a);
    else k_init<float><<<nblk, INIT_TPB, 0, s>>>(static_cast<float*>(Q), a);
    return cudaGetLastError();
}
}  // namespace hermes

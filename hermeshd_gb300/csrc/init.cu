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

namespace hermes {
// per box: the sum of its chunks' partial sums, in chunk order, times the cell volume
__global__ void __launch_bounds__(32) k_cons_final(ConsArgs a) {
    const int bx = blockIdx.x, v = threadIdx.x;
    if (v >= 5) return;
    const Box& B = a.boxes[bx];
    const double vol = 1.0 / (B.di[0] * B.di[1] * B.di[2]);
    double s = 0.0;
    for (int ch = a.box_chunk0[bx]; ch < a.box_chunk0[bx + 1]; ++ch) s += a.partial[5 * ch + v];
    a.out[5 * bx + v] = s * vol;
}

cudaError_t cons_launch(int precision, const void* Q, const ConsArgs& a, int nbox, cudaStream_t s) {
    if (a.nchunk <= 0) return cudaSuccess;
    if (precision == 64) k_cons_partial<double><<<a.nchunk, CONS_TPB, 0, s>>>(static_cast<const double*>(Q), a);
    else k_cons_partial<float><<<a.nchunk, CONS_TPB, 0, s>>>(static_cast<const float*>(Q), a);
    k_cons_final<<<nbox, 32, 0, s>>>(a);
    return cudaGetLastError();
}
}  // namespace hermes

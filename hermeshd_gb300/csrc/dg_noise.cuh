// dg_noise.cuh -- the stochastic stress (random.f90:106-145, Philox-4x32-10
// counters of dg_physics.cuh) drawn by kernels of its own and staged in HBM
// for the face and cell kernels of a stage.
//
// Drawn inside k_face / k_cell, the generator shares their registers and,
// in k_cell, runs on the hydro half of each cell's thread pair only, so the
// draws are latency-bound; here every draw is one thread of a full-occupancy
// kernel, and the consumers read 6 values per point.  The counters are the
// same, so the staged and the inline draws are the same numbers.
//   k_noise_cell  thread per (cell, direction, quadrature point), the
//                 (direction, point) pair in blockIdx.y (no 64-bit division): the
//                 interior stress of flux call kind 3 + d, written as
//                 [d][point][component][cell]
//   k_noise_face  thread per (face, point, side) of one direction: the two
//                 per-side stresses of the face call, written as
//                 [side][component][point][face] after the faces of the
//                 directions before it
#pragma once

#include "dg_kernels.cuh"

namespace hermes {

constexpr int NOISE_TPB = 256;

struct NoiseArgs {
    Geom G;
    Phys ph;
    const unsigned long long* step;
    unsigned stage;
};

// grid (cells / NOISE_TPB, 3 NPG): blockIdx.y = d * NPG + g
template <class T, class TB>
__global__ void __launch_bounds__(NOISE_TPB) k_noise_cell(T* __restrict__ out, NoiseArgs a) {
    pdl_enter();
    const long long ncl = a.G.ncell;
    const long long gc = (long long)blockIdx.x * NOISE_TPB + threadIdx.x;
    if (gc >= ncl) return;
    const int r = blockIdx.y;
    const int d = r / TB::NPG, g = r % TB::NPG;
    const int bx = box_of_cell(a.G, gc);
    const Box& B = a.G.boxes[bx];
    T S[6];
    random_stress<T>(a.ph, B.seed, NoiseCtr{*a.step, a.stage}, 3 + d, (unsigned long long)(gc - B.cell0), g, S);
#pragma unroll
    for (int c = 0; c < 6; ++c) out[((long long)r * 6 + c) * ncl + gc] = S[c];
}

// grid (faces / NOISE_TPB, 2 NF): blockIdx.y = side * NF + P
template <class T, class TB, int DIR>
__global__ void __launch_bounds__(NOISE_TPB) k_noise_face(T* __restrict__ out, NoiseArgs a) {
    pdl_enter();
    const long long nfa = a.G.nface[DIR];
    const long long gf = (long long)blockIdx.x * NOISE_TPB + threadIdx.x;
    if (gf >= nfa) return;
    const int r = blockIdx.y;
    const int P = r % TB::NF, side = r / TB::NF;
    const int bx = box_of_face<DIR>(a.G, gf);
    const Box& B = a.G.boxes[bx];
    T S[6];
    random_stress<T>(a.ph, B.seed, NoiseCtr{*a.step, a.stage}, DIR, (unsigned long long)(gf - B.face0[DIR]),
                     (unsigned)(P + side * TB::NF), S);
    T* base = out + 12ll * TB::NF * a.G.face0_dir[DIR];
#pragma unroll
    for (int c = 0; c < 6; ++c) base[((long long)(side * 6 + c) * TB::NF + P) * nfa + gf] = S[c];
}

// the interior draws into cellbuf and the face draws into facebuf (a null
// buffer skips its kernels)
template <class T, int NB, int NQD>
cudaError_t noise_launch(void* cellbuf, void* facebuf, const NoiseArgs& a, cudaStream_t s) {
    using TB = hermes_tab::Tab<NB, NQD>;
    auto blocks = [](long long n) { return (unsigned)((n + NOISE_TPB - 1) / NOISE_TPB); };
    if (cellbuf && a.G.ncell > 0)
        launch_k(a.G.pdl, k_noise_cell<T, TB>, dim3(blocks(a.G.ncell), 3 * TB::NPG), NOISE_TPB, 0, s,
                 static_cast<T*>(cellbuf), a);
    if (!facebuf) return cudaGetLastError();
    if (a.G.nface[0] > 0)
        launch_k(a.G.pdl, k_noise_face<T, TB, 0>, dim3(blocks(a.G.nface[0]), 2 * TB::NF), NOISE_TPB, 0, s,
                 static_cast<T*>(facebuf), a);
    if (a.G.nface[1] > 0)
        launch_k(a.G.pdl, k_noise_face<T, TB, 1>, dim3(blocks(a.G.nface[1]), 2 * TB::NF), NOISE_TPB, 0, s,
                 static_cast<T*>(facebuf), a);
    if (a.G.nface[2] > 0)
        launch_k(a.G.pdl, k_noise_face<T, TB, 2>, dim3(blocks(a.G.nface[2]), 2 * TB::NF), NOISE_TPB, 0, s,
                 static_cast<T*>(facebuf), a);
    return cudaGetLastError();
}

using NoiseFn = cudaError_t (*)(void*, void*, const NoiseArgs&, cudaStream_t);
bool noise_launcher(int precision, int nb, NoiseFn* out);

}  // namespace hermes

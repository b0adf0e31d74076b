// dg_noise.cuh -- the stochastic stress (random.f90:106-145, Philox-4x32-10
// counters of dg_physics.cuh) drawn by kernels of its own and staged in HBM
// for the face and cell kernels of a stage.
//
// Drawn inside k_face / k_cell, the generator shares their registers and,
// in k_cell, runs on the hydro half of each cell's thread pair only, so the
// draws are latency-bound; here every draw is one thread of a full-occupancy
// kernel, and the consumers read 6 values per point.  The counters are the
// same, so the staged and the inline draws are the same numbers.
//   k_noise_cell  thread per (cell, direction, quadrature point): the
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

template <class T, class TB>
__global__ void __launch_bounds__(NOISE_TPB) k_noise_cell(T* __restrict__ out, NoiseArgs a) {
    const long long ncl = a.G.ncell;
    const long long idx = (long long)blockIdx.x * NOISE_TPB + threadIdx.x;
    if (idx >= ncl * 3 * TB::NPG) return;
    const long long gc = idx % ncl;
    const int r = (int)(idx / ncl);                 // d * NPG + g
    const int d = r / TB::NPG, g = r % TB::NPG;
    const int bx = find_box(a.G.boxes, a.G.nbox, gc, [](const Box& b) { return b.cell0; });
    const Box& B = a.G.boxes[bx];
    T S[6];
    random_stress<T>(a.ph, B.seed, NoiseCtr{*a.step, a.stage}, 3 + d, (unsigned long long)(gc - B.cell0), g, S);
#pragma unroll
    for (int c = 0; c < 6; ++c) out[((long long)r * 6 + c) * ncl + gc] = S[c];
}

template <class T, class TB, int DIR>
__global__ void __launch_bounds__(NOISE_TPB) k_noise_face(T* __restrict__ out, NoiseArgs a) {
    const long long nfa = a.G.nface[DIR];
    const long long idx = (long long)blockIdx.x * NOISE_TPB + threadIdx.x;
    if (idx >= nfa * 2 * TB::NF) return;
    const long long gf = idx % nfa;
    const int r = (int)(idx / nfa);                 // side * NF + P
    const int P = r % TB::NF, side = r / TB::NF;
    const int bx = find_box(a.G.boxes, a.G.nbox, gf, [](const Box& b) { return b.face0[DIR]; });
    const Box& B = a.G.boxes[bx];
    T S[6];
    random_stress<T>(a.ph, B.seed, NoiseCtr{*a.step, a.stage}, DIR, (unsigned long long)(gf - B.face0[DIR]),
                     (unsigned)(P + side * TB::NF), S);
    T* base = out + 12ll * TB::NF * a.G.face0_dir[DIR];
#pragma unroll
    for (int c = 0; c < 6; ++c) base[((long long)(side * 6 + c) * TB::NF + P) * nfa + gf] = S[c];
}

template <class T, int NB, int NQD>
cudaError_t noise_launch(void* cellbuf, void* facebuf, const NoiseArgs& a, cudaStream_t s) {
    using TB = hermes_tab::Tab<NB, NQD>;
    const long long nc = a.G.ncell * 3 * TB::NPG;
    if (nc > 0) k_noise_cell<T, TB><<<(unsigned)((nc + NOISE_TPB - 1) / NOISE_TPB), NOISE_TPB, 0, s>>>(static_cast<T*>(cellbuf), a);
    const long long n0 = a.G.nface[0] * 2 * TB::NF, n1 = a.G.nface[1] * 2 * TB::NF, n2 = a.G.nface[2] * 2 * TB::NF;
    if (n0 > 0) k_noise_face<T, TB, 0><<<(unsigned)((n0 + NOISE_TPB - 1) / NOISE_TPB), NOISE_TPB, 0, s>>>(static_cast<T*>(facebuf), a);
    if (n1 > 0) k_noise_face<T, TB, 1><<<(unsigned)((n1 + NOISE_TPB - 1) / NOISE_TPB), NOISE_TPB, 0, s>>>(static_cast<T*>(facebuf), a);
    if (n2 > 0) k_noise_face<T, TB, 2><<<(unsigned)((n2 + NOISE_TPB - 1) / NOISE_TPB), NOISE_TPB, 0, s>>>(static_cast<T*>(facebuf), a);
    return cudaGetLastError();
}

using NoiseFn = cudaError_t (*)(void*, void*, const NoiseArgs&, cudaStream_t);
bool noise_launcher(int precision, int nb, NoiseFn* out);

}  // namespace hermes

// dg_trace.cuh -- k_trace: the face traces of every cell, evaluated once per
// cell, direction and variable and stored for the face kernels (FP64 path, nbasis 8
// and 10, where the FP64 pipe bounds the step and the trace sums are the
// largest part of a face point's arithmetic).
//
// A face point's trace is sum_b phi_b(P) Q(b, v) (flux.f90:217,230).  Both
// faces of one direction share the tangential coordinates of their points,
// and the face tables are mirror-symmetric in the normal coordinate and in
// the second tangential one (face point p = i*NE + m, mirror m -> NE-1-m):
// the values at a mirror pair of points on both faces are four signed sums
// of four partial sums, one per parity class (normal, tangential) of the
// basis functions.  Each table product is done once for up to four values.
//
// Layout of the buffer: [direction][side (0 minus, 1 plus)][variable][point]
// [cell of the whole grid], so the face kernel's loads of consecutive faces
// are consecutive cells.
#pragma once

#include "dg_kernels.cuh"

namespace hermes {

constexpr int TRACE_TPB = 128;

// the traces of variable v of one cell on both faces of direction DIR
template <class T, class TB, int DIR>
__device__ __forceinline__ void trace_cell(const T* __restrict__ Qb, long long nc, long long le, int v,
                                           T* __restrict__ tr, long long ncl, long long gc) {
    using FO = FOrbit<TB>;
    static_assert(face_tables_symmetric<TB, DIR, false>(), "face tables not mirror-symmetric");
    constexpr int NF = TB::NF;
    T* t1 = tr + (long long)((DIR * 2 + 1) * NQ) * NF * ncl + gc;   // plus face
    T* t0 = tr + (long long)((DIR * 2 + 0) * NQ) * NF * ncl + gc;   // minus face
    T q[TB::NB];
#pragma unroll
    for (int b = 0; b < TB::NB; ++b) q[b] = __ldg(Qb + (long long)(b * NQ + v) * nc + le);
    sfor<FO::NCH>([&](auto cc) {
        constexpr int c = decltype(cc)::value;
        T S[4] = {T(0), T(0), T(0), T(0)};
        sfor<TB::NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            constexpr int k = face_class<TB, DIR, false>(c, b);
            if constexpr (k >= 0) S[k] = fma(T(ftab<TB, DIR, 1>(FO::pA(c), b)), q[b], S[k]);
        });
        constexpr bool h0 = face_has<TB, DIR, false>(c, 0), h1 = face_has<TB, DIR, false>(c, 1);
        constexpr bool h2 = face_has<TB, DIR, false>(c, 2), h3 = face_has<TB, DIR, false>(c, 3);
        // normal-even / normal-odd parts at pA (tangential classes summed) and at pB
        const T A0 = sum_opt<h0, h2>(S[0], S[2]), A1 = sum_opt<h1, h3>(S[1], S[3]);
        constexpr bool hA0 = h0 || h2, hA1 = h1 || h3;
        const long long oA = ((long long)v * NF + FO::pA(c)) * ncl;
        t1[oA] = sum_opt<hA0, hA1>(A0, A1);
        t0[oA] = diff_opt<hA0, hA1>(A0, A1);
        if constexpr (FO::pair(c)) {
            const T B0 = diff_opt<h0, h2>(S[0], S[2]), B1 = diff_opt<h1, h3>(S[1], S[3]);
            const long long oB = ((long long)v * NF + FO::pB(c)) * ncl;
            t1[oB] = sum_opt<hA0, hA1>(B0, B1);
            t0[oB] = diff_opt<hA0, hA1>(B0, B1);
        }
    });
}

// thread per (cell, direction, variable) for the variables v0 .. v0+nv-1;
// grid (cells / TRACE_TPB, 3 nv): blockIdx.y = direction * nv + variable - v0
template <class T, class TB>
__global__ void __launch_bounds__(TRACE_TPB) k_trace(const T* __restrict__ Q, T* __restrict__ tr, Geom G, int v0, int nv) {
    pdl_enter();
    const long long gc = (long long)blockIdx.x * TRACE_TPB + threadIdx.x;
    if (gc >= G.ncell) return;
    const int bx = box_of_cell(G, gc);
    const Box& B = G.boxes[bx];
    const T* Qb = Q + B.q0;
    const long long le = gc - B.cell0;
    const int d = blockIdx.y / nv, v = v0 + blockIdx.y % nv;
    if (d == 0) trace_cell<T, TB, 0>(Qb, B.ncell, le, v, tr, G.ncell, gc);
    else if (d == 1) trace_cell<T, TB, 1>(Qb, B.ncell, le, v, tr, G.ncell, gc);
    else trace_cell<T, TB, 2>(Qb, B.ncell, le, v, tr, G.ncell, gc);
}

}  // namespace hermes

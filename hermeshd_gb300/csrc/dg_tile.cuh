// dg_tile.cuh -- k_tile: one whole SSP-RK stage of the linear basis (nbasis 4,
// iquad 2) in one kernel, and k_mindt_limit, the CFL reduction fused with the
// first stage's positivity limiter.
//
// A block owns a tile of cells of one box (8 x 8 x 4 = 256 cells, one thread
// per cell) and, per stage:
//   1. for each direction: the numerical fluxes at every face point of the
//      tile's faces (flux.f90:197-450: traces of both cells, boundary ghosts of
//      boundary.f90:40-338, point fluxes, central/LLF, HLLC or Roe, the
//      stochastic stress of the face call drawn in place), kept in shared
//      memory, and each cell's surface sums of that direction (flux.f90:958-978)
//      added to its right-hand side, also in shared memory;
//   2. the volume quadrature at the cell's interior points with the interior
//      stochastic stress drawn in place (flux.f90:751-928), the linear sources
//      (sources.f90:36-70), the forward-Euler update with the semi-implicit
//      relaxation of ivis 1 and the RK combination (integrator.f90:62-178), the
//      NaN check of the cell averages (integrator.f90:234-250) and, for a stage
//      whose output is the next stage's input, that stage's positivity limiter
//      (flux.f90:1077-1164, applied in place at the start of euler_step by the
//      reference) -- then one store of the cell's coefficients.
// So a stage reads the coefficient field once (each cell by its own tile and,
// for the tile-boundary faces, by the neighbouring tile) and writes it once;
// face fluxes and noise never leave the SM.  A face on a tile boundary is
// evaluated by both tiles that share it, from the same inputs and the same
// Philox counters, so both see the same bits.
//
// The stage output must not alias its input (other tiles read the input as
// their halo while this tile writes): the step keeps a third state buffer.
#pragma once

#include "dg_kernels.cuh"

namespace hermes {

constexpr int TILE_NT = 256;          // threads (= cells) per tile
constexpr int TILE_X = 8, TILE_Y = 8, TILE_Z = 4;

struct TileArgs {
    CellArgs c;                // geometry, physics, dt per box, noise counter, flags, stage, mode, comb
    const long long* tile0;    // first tile of each box in the launch, nbox + 1 entries
    int fmax;                  // face-flux buffer entries per (variable, point): the largest face count of a direction
    int limit_out;             // apply the next stage's positivity limiter to the output
};

// the entry of a compile-time table column at a row chosen at run time: the
// constant where the column is constant, a sign select where its entries are
// +-c (the tensor Legendre tables at symmetric Gauss points), else a select
// chain over the rows' constants (converted to T at compile time)
template <int NROW, class Tab>
__host__ __device__ constexpr bool column_any(Tab tab) {
    for (int r = 0; r < NROW; ++r)
        if (tab(r) != 0.0) return true;
    return false;
}
template <int NROW, class Tab>
__host__ __device__ constexpr bool column_constant(Tab tab) {
    for (int r = 1; r < NROW; ++r)
        if (tab(r) != tab(0)) return false;
    return true;
}
template <int NROW, class Tab>
__host__ __device__ constexpr bool column_pm(Tab tab) {
    for (int r = 1; r < NROW; ++r)
        if (tab(r) != tab(0) && tab(r) != -tab(0)) return false;
    return NROW <= 32;
}
template <int NROW, class Tab>
__host__ __device__ constexpr unsigned column_sign_mask(Tab tab) {
    unsigned m = 0;
    for (int r = 0; r < NROW; ++r)
        if (tab(r) == tab(0)) m |= 1u << r;
    return m;
}
template <int NROW, class T, class Tab>
__device__ __forceinline__ T rt_entry(int r, Tab tab) {
    if constexpr (column_constant<NROW>(tab)) {
        return T(tab(0));
    } else if constexpr (column_pm<NROW>(tab)) {
        constexpr unsigned m = column_sign_mask<NROW>(tab);
        return ((m >> r) & 1u) ? T(tab(0)) : T(-tab(0));
    } else {
        T c = T(0);
        sfor<NROW>([&](auto rr) {
            if (r == decltype(rr)::value) c = T(tab(decltype(rr)::value));
        });
        return c;
    }
}

// trace of all variables of one cell at a face point chosen at run time
template <class TB, int DIR, int SIDE, class T>
__device__ __forceinline__ void trace_rt(const T* __restrict__ Qb, long long nc, long long cell, int P, T q[NQ]) {
    sfor<TB::NF>([&](auto pp) {
        if (P == decltype(pp)::value) trace_pt<TB, DIR, SIDE, decltype(pp)::value>(Qb, nc, cell, q);
    });
}

// the numerical flux at face point P of the face with coordinates fc (the
// DIR coordinate is the face plane 0..n) of box B, scaled by the inverse
// spacing: the same operations as face_point (dg_kernels.cuh), with the
// point chosen at run time and the stochastic stress drawn in place.  Args:
// CellArgs or FaceArgs (ph, step, stage)
template <class T, class TB, int DIR, bool NOISE, class Args>
__device__ __forceinline__ void tile_face_flux(const T* __restrict__ Q, const Args& a, const Box& B, const int fc[3],
                                               int P, T F[NQ]) {
    const Phys& ph = a.ph;
    constexpr int NF = TB::NF;
    const int n0 = B.n[0], n1 = B.n[1];
    const int n = B.n[DIR];
    const bool dedup = B.nfp[DIR] == n;                    // both ends periodic: n planes, plane n is plane 0
    int s = fc[DIR];
    if (dedup && s == n) s = 0;
    const int i = DIR == 0 ? s : fc[0], j = DIR == 1 ? s : fc[1], k = DIR == 2 ? s : fc[2];
    const int ex = DIR == 0 ? B.nfp[0] : n0, ey = DIR == 1 ? B.nfp[1] : n1;
    const long long lf = (long long)i + (long long)ex * (j + (long long)ey * k);
    const T* Qb = Q + B.q0;
    const long long nc = B.ncell;
    auto cell_at = [&](int c) -> long long {
        const int ci = DIR == 0 ? c : i, cj = DIR == 1 ? c : j, ck = DIR == 2 ? c : k;
        return (long long)ci + (long long)n0 * (cj + (long long)n1 * ck);
    };
    constexpr int MN = DIR == 0 ? MX : DIR == 1 ? MY : MZ;   // normal momentum
    T qL[NQ], qR[NQ];
    if (dedup || (s > 0 && s < n)) {
        const int lo = s > 0 ? s - 1 : n - 1;
        trace_rt<TB, DIR, 1>(Qb, nc, cell_at(lo), P, qL);
        trace_rt<TB, DIR, 0>(Qb, nc, cell_at(s), P, qR);
    } else if (s == 0) {
        // low boundary: ghost from the first cell's minus trace (boundary.f90:40-244)
        const long long c0 = cell_at(0);
        trace_rt<TB, DIR, 0>(Qb, nc, c0, P, qR);
        const int code = B.bc[2 * DIR];
        if (code == BC_PERIODIC) {
            for (int v = 0; v < NQ; ++v) qL[v] = T(0);
        } else {
            for (int v = 0; v < NQ; ++v) qL[v] = qR[v];
            if (DIR == 0 && code == BC_INFLOW) {
                // boundary.f90:568-612
                const double lyd = -(ph.inflow_ly / 2.0);
                const double yc = lyd + (j + 0.5) * (1.0 / B.di[1]);
                const double yp = yc - lyd;
                const double vx = 4 * ph.inflow_u * yp * (ph.inflow_ly - yp) / (ph.inflow_ly * ph.inflow_ly);
                const double den = ph.inflow_rho;
                qL[RH] = T(den);
                qL[MX] = T(den * vx);
                qL[MY] = T(0);
                qL[MZ] = T(0);
                qL[EN] = T(ph.inflow_p / ph.aindm1 + 0.5 * den * (vx * vx));
            }
            if (code == BC_NOSLIP) { qL[MX] = T(0); qL[MY] = T(0); qL[MZ] = T(0); }
            else if (code == BC_WALL) { qL[MN] = T(0); }
            else if (code == BC_OUTFLOW) {
                T mmax = -T(INFINITY);
                sfor<NF>([&](auto pp) { mmax = fmax(mmax, trace_var<TB, DIR, 0, decltype(pp)::value, MN>(Qb, nc, c0)); });
                if (mmax > T(0)) qL[MN] = T(0);
            }
        }
    } else {
        // high boundary (s == n)
        const long long cl = cell_at(n - 1);
        trace_rt<TB, DIR, 1>(Qb, nc, cl, P, qL);
        const int code = B.bc[2 * DIR + 1];
        if (code == BC_PERIODIC) {
            trace_rt<TB, DIR, 0>(Qb, nc, cell_at(0), P, qR);
        } else if (code == BC_OUTFLOW && DIR == 0) {
            for (int v = 0; v < NQ; ++v) qR[v] = T(0);
        } else {
            for (int v = 0; v < NQ; ++v) qR[v] = qL[v];
            if (code == BC_NOSLIP) { qR[MX] = T(0); qR[MY] = T(0); qR[MZ] = T(0); }
            else if (code == BC_WALL) { qR[MN] = T(0); }
            else if (code == BC_OUTFLOW) {
                T mmin = T(INFINITY);
                sfor<NF>([&](auto pp) { mmin = fmin(mmin, trace_var<TB, DIR, 1, decltype(pp)::value, MN>(Qb, nc, cl)); });
                if (mmin < T(0)) qR[MN] = T(0);
            }
        }
    }
    T SL[6] = {T(0), T(0), T(0), T(0), T(0), T(0)}, SR[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
    if constexpr (NOISE) {
        if (ph.llns) {
            // the two per-side stresses of the face call (k_noise_face's
            // counters); one copy of the generator for both sides
            const NoiseCtr nctr{*a.step, a.stage};
#pragma unroll 1
            for (int side = 0; side < 2; ++side) {
                T S6[6];
                random_stress<T>(ph, B.seed, nctr, DIR, (unsigned long long)lf, (unsigned)(P + side * NF), S6);
                if (side == 0) {
#pragma unroll
                    for (int c = 0; c < 6; ++c) SL[c] = S6[c];
                } else {
#pragma unroll
                    for (int c = 0; c < 6; ++c) SR[c] = S6[c];
                }
            }
        }
    }
    T rho_i_last = T(0);
    if (ph.ihllc == 1 && ph.ieos == 2) {
        // 1/rho of the last point of the reference's call: the right state at point NF-1
        T rlast;
        if (dedup || s < n) rlast = trace_var<TB, DIR, 0, NF - 1, RH>(Qb, nc, cell_at(s));
        else if (B.bc[2 * DIR + 1] == BC_PERIODIC) rlast = trace_var<TB, DIR, 0, NF - 1, RH>(Qb, nc, cell_at(0));
        else if (B.bc[2 * DIR + 1] == BC_OUTFLOW && DIR == 0) rlast = T(0);
        else rlast = trace_var<TB, DIR, 1, NF - 1, RH>(Qb, nc, cell_at(n - 1));
        rho_i_last = T(1) / rlast;
    }
    face_flux_fn<T, DIR>(ph, qL, qR, SL, SR, rho_i_last, F, T(B.di[DIR]));
}

// k_face_pl: the face fluxes of one direction, one thread per face looping
// over the face's points at run time (blockIdx.y = 1).  Only the trace
// evaluation is instantiated per point, so the body exists once (the point
// per block of k_face instantiates it NF times) and the face's set-up (box,
// coordinates, boundary kind) is done once for its points.  The stochastic
// stress is drawn in place; the same operations as k_face, so the same bits.
template <class T, class TB, int DIR, bool NOISE>
__global__ void __launch_bounds__(FACE_TPB, (FaceMinBlocks<T>::value)) k_face_pl(const T* __restrict__ Q, T* __restrict__ flux,
                                                                              FaceArgs a) {
    pdl_enter();
    const long long gf = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gf >= a.G.nface[DIR]) return;
    const int bx = box_of_face<DIR>(a.G, gf);
    const Box& B = a.G.boxes[bx];
    const long long lf = gf - B.face0[DIR];
    const int ex = DIR == 0 ? B.nfp[0] : B.n[0], ey = DIR == 1 ? B.nfp[1] : B.n[1];
    const unsigned lfu = (unsigned)lf, t = lfu / (unsigned)ex;   // fewer than 2^31 faces per box
    const int fc[3] = {(int)(lfu - t * (unsigned)ex), (int)(t % (unsigned)ey), (int)(t / (unsigned)ey)};
    const long long nfd = (long long)ex * ey * (DIR == 2 ? B.nfp[2] : B.n[2]);
    T* fb = flux + B.fbase[DIR];
#pragma unroll 1
    for (int P = 0; P < TB::NF; ++P) {
        T F[NQ];
        tile_face_flux<T, TB, DIR, NOISE>(Q, a, B, fc, P, F);
#pragma unroll
        for (int v = 0; v < NQ; ++v) fb[(long long)(v * TB::NF + P) * nfd + lf] = F[v];
    }
}

// resident tiles per SM: one (no register cap: at two per SM, FP32's 128
// registers spilled ~300 B per thread to L2)
template <class T>
struct TileMinBlocks {
    static constexpr int value = 1;
};

// shared memory of a tile: the face fluxes of one direction, [NQ][NF][fmax],
// then the right-hand-side accumulators, [NQ * NB][TILE_NT]
template <class T, class TB>
__host__ __device__ constexpr size_t tile_smem(int fmax) {
    return ((size_t)NQ * TB::NF * fmax + (size_t)NQ * TB::NB * TILE_NT) * sizeof(T);
}

// the positivity limiter of k_limit (same fast path, same operations) on the
// rh..en rows of one cell held in registers; FP32 evaluates near the floors in FP64
template <class T, class TB>
__device__ __forceinline__ void limit_rows(const Phys& ph, T (&o)[NQ][TB::NB]) {
    constexpr int NB = TB::NB;
    T q[5][NB];
    sfor<5>([&](auto vv) { sfor<NB>([&](auto bb) { q[decltype(vv)::value][decltype(bb)::value] = o[decltype(vv)::value][decltype(bb)::value]; }); });
    if (q[RH][0] >= PHC(T, ph, rh_floor) && limit_bound_clear<TB, T>(ph, q)) return;
    if constexpr (std::is_same<T, double>::value) {
        if (!limit_cell<TB, double>(ph, q)) return;
    } else {
        double qd[5][NB];
        sfor<5>([&](auto vv) { sfor<NB>([&](auto bb) { qd[decltype(vv)::value][decltype(bb)::value] = (double)q[decltype(vv)::value][decltype(bb)::value]; }); });
        if (!limit_cell<TB, double>(ph, qd)) return;
        sfor<5>([&](auto vv) { sfor<NB>([&](auto bb) { q[decltype(vv)::value][decltype(bb)::value] = (T)qd[decltype(vv)::value][decltype(bb)::value]; }); });
    }
    sfor<5>([&](auto vv) { sfor<NB>([&](auto bb) { o[decltype(vv)::value][decltype(bb)::value] = q[decltype(vv)::value][decltype(bb)::value]; }); });
}

// every basis function has a volume term along at most one direction (true
// of the linear basis), so folding one direction's terms at a time into the
// right-hand side gives the same sums as one accumulation over directions
template <class TB>
__host__ __device__ constexpr bool volume_terms_one_direction() {
    for (int b = 0; b < TB::NB; ++b) {
        int dirs = 0;
        bool x = false, y = false, z = false;
        for (int g = 0; g < TB::NPG; ++g) {
            x = x || TB::VX(g, b) != 0.0;
            y = y || TB::VY(g, b) != 0.0;
            z = z || TB::VZ(g, b) != 0.0;
        }
        dirs = (x ? 1 : 0) + (y ? 1 : 0) + (z ? 1 : 0);
        if (dirs > 1) return false;
    }
    return true;
}

// grid: one block per tile of every box (ta.tile0), TILE_NT threads, dynamic
// shared memory tile_smem<T, TB>(ta.fmax).  ivis 0 and 1 only (the linear
// stress fluxes and sources); Qin must not alias out (Q0 may: each thread
// reads its own cell's Q0 before writing it).
template <class T, class TB, bool NOISE>
__global__ void __launch_bounds__(TILE_NT, (TileMinBlocks<T>::value))
    k_tile(const T* __restrict__ Qin, const T* Q0, T* out, TileArgs ta) {
    pdl_enter();
    constexpr int NB = TB::NB, NF = TB::NF;
    static_assert(volume_terms_one_direction<TB>(), "the fused stage folds the volume terms one direction at a time");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const CellArgs& a = ta.c;
    const Phys& ph = a.ph;
    const int fmax = ta.fmax;
    T* Fs = reinterpret_cast<T*>(smem_raw);             // [NQ][NF][fmax]
    T* rs = Fs + (size_t)NQ * NF * fmax;                 // [NQ * NB][TILE_NT]
    const int tid = threadIdx.x;
    // the tile: box (binary search over the first tiles) and its place in the box
    const long long t = blockIdx.x;
    int bx = 0;
    {
        int lo = 0, hi = a.G.nbox - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (ta.tile0[mid] <= t) lo = mid; else hi = mid - 1;
        }
        bx = lo;
    }
    const Box& B = a.G.boxes[bx];
    const int ntx = (B.n[0] + TILE_X - 1) / TILE_X, nty = (B.n[1] + TILE_Y - 1) / TILE_Y;
    const int lt = (int)(t - ta.tile0[bx]);
    const int o[3] = {(lt % ntx) * TILE_X, ((lt / ntx) % nty) * TILE_Y, (lt / (ntx * nty)) * TILE_Z};
    const int lx = tid % TILE_X, ly = (tid / TILE_X) % TILE_Y, lz = tid / (TILE_X * TILE_Y);
    const int ci = o[0] + lx, cj = o[1] + ly, ck = o[2] + lz;
    const bool act = ci < B.n[0] && cj < B.n[1] && ck < B.n[2];
    const long long nc = B.ncell;
    const long long le = act ? (long long)ci + (long long)B.n[0] * (cj + (long long)B.n[1] * ck) : 0;
#pragma unroll
    for (int m = 0; m < NQ * NB; ++m) rs[m * TILE_NT + tid] = T(0);

    // ---- faces and surface sums, one direction at a time
    sfor<3>([&](auto dd) {
        constexpr int D = decltype(dd)::value;
        constexpr int E0 = TILE_X + (D == 0), E1 = TILE_Y + (D == 1), E2 = TILE_Z + (D == 2);
        constexpr int NFL = E0 * E1 * E2;               // faces of the tile in direction D
#pragma unroll 1
        for (int it = tid; it < NF * NFL; it += TILE_NT) {
            const int P = it / NFL, fl = it - P * NFL;
            const int fc[3] = {o[0] + fl % E0, o[1] + (fl / E0) % E1, o[2] + fl / (E0 * E1)};
            const bool ok = (D == 0 ? fc[0] <= B.n[0] : fc[0] < B.n[0]) && (D == 1 ? fc[1] <= B.n[1] : fc[1] < B.n[1]) &&
                            (D == 2 ? fc[2] <= B.n[2] : fc[2] < B.n[2]);
            T F[NQ];
            if (ok) {
                tile_face_flux<T, TB, D, NOISE>(Qin, a, B, fc, P, F);
            } else {
#pragma unroll
                for (int v = 0; v < NQ; ++v) F[v] = T(0);
            }
#pragma unroll
            for (int v = 0; v < NQ; ++v) Fs[(size_t)(v * NF + P) * fmax + fl] = F[v];
        }
        __syncthreads();
        if (act) {
            // the cell's minus face has its local coordinates, the plus face one more along D
            const int fm = lx + E0 * (ly + E1 * lz);
            const int fp = fm + (D == 0 ? 1 : D == 1 ? E0 : E0 * E1);
            static_assert(face_tables_symmetric<TB, D, true>(), "surface tables not mirror-symmetric");
            sfor<NQ>([&](auto vv) {
                constexpr int v = decltype(vv)::value;
                T r[NB];
                sfor<NB>([&](auto bb) { r[decltype(bb)::value] = rs[(v * NB + decltype(bb)::value) * TILE_NT + tid]; });
                sfor<NF>([&](auto pp) {
                    constexpr int p = decltype(pp)::value;
                    const T Fp = Fs[(size_t)(v * NF + p) * fmax + fp];
                    const T Fm = Fs[(size_t)(v * NF + p) * fmax + fm];
                    const T Fsum = Fp + Fm, Fdif = Fp - Fm;
                    sfor<NB>([&](auto bb) {
                        constexpr int b = decltype(bb)::value;
                        constexpr double cp = stab<TB, D, 1>(p, b), cm = stab<TB, D, 0>(p, b);
                        if constexpr (cp != 0.0) r[b] = fma(T(cp), cm == cp ? Fsum : Fdif, r[b]);
                    });
                });
                sfor<NB>([&](auto bb) { rs[(v * NB + decltype(bb)::value) * TILE_NT + tid] = r[decltype(bb)::value]; });
            });
        }
        __syncthreads();
    });
    if (!act) return;

    // ---- volume quadrature, sources, update, RK combination, limiter, store
    const T* Qb = Qin + B.q0;
    T q[NQ][NB];
    sfor<NQ>([&](auto vv) {
        sfor<NB>([&](auto bb) {
            constexpr int v = decltype(vv)::value, b = decltype(bb)::value;
            q[v][b] = Qb[(long long)(b * NQ + v) * nc + le];
        });
    });
    const T di[3] = {T(B.di[0]), T(B.di[1]), T(B.di[2])};
    // the interior stresses of one direction, drawn for all points of the
    // cell before its flux loop (k_noise_cell's counters), into the face-flux
    // buffer, which the face phase no longer needs: [point][component][TILE_NT]
    T* Ns = Fs;
    sfor<3>([&](auto dd) {
        constexpr int d = decltype(dd)::value;
        // the volume terms of direction d (its own accumulators, folded into
        // the column after the direction: a basis function whose derivative
        // along d is the only nonzero one gets the same sum either way)
        T acc[NQ][NB];
        sfor<NQ>([&](auto vv) { sfor<NB>([&](auto bb) { acc[decltype(vv)::value][decltype(bb)::value] = T(0); }); });
        if constexpr (NOISE) {
            if (ph.llns) {
                const NoiseCtr nctr{*a.step, a.stage};
#pragma unroll 1
                for (int g = 0; g < TB::NPG; ++g) {
                    T S6[6];
                    random_stress<T>(ph, B.seed, nctr, 3 + d, (unsigned long long)le, (unsigned)g, S6);
#pragma unroll
                    for (int c = 0; c < 6; ++c) Ns[(g * 6 + c) * TILE_NT + tid] = S6[c];
                }
            }
        }
        // one loop body for every interior point (table entries selected at
        // run time), which bounds the live registers to one point's values
#pragma unroll 1
        for (int g = 0; g < TB::NPG; ++g) {
            T u[NQ];
            T cint[NB];
            sfor<NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                cint[b] = rt_entry<TB::NPG, T>(g, [](int r) { return TB::INT(r, b); });
            });
            sfor<NQ>([&](auto vv) {
                constexpr int v = decltype(vv)::value;
                T s = T(0);
                sfor<NB>([&](auto bb) {
                    constexpr int b = decltype(bb)::value;
                    if constexpr (column_any<TB::NPG>([](int r) { return TB::INT(r, b); })) s = fma(cint[b], q[v][b], s);
                });
                u[v] = s;
            });
            const Prim<T> w = primitives(ph, u);
            T S[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
            if constexpr (NOISE) {
                if (ph.llns) {
#pragma unroll
                    for (int c = 0; c < 6; ++c) S[c] = Ns[(g * 6 + c) * TILE_NT + tid];
                }
            }
            T f[NQ];
            point_flux<T, d>(ph, u, w, S, f);
            sfor<NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                if constexpr (vtab_any<TB, d>(b)) {
                    const T cv = rt_entry<TB::NPG, T>(g, [](int r) { return vtab<TB, d>(r, b); });
                    sfor<NQ>([&](auto vv) {
                        constexpr int v = decltype(vv)::value;
                        acc[v][b] = fma(cv, f[v] * di[d], acc[v][b]);
                    });
                }
            });
        }
        sfor<NQ>([&](auto vv) { sfor<NB>([&](auto bb) {
            constexpr int v = decltype(vv)::value, b = decltype(bb)::value;
            if constexpr (vtab_any<TB, d>(b)) rs[(v * NB + b) * TILE_NT + tid] -= acc[v][b];
        }); });
    });
    // glflux - source into the accumulator column, with the linear sources:
    // the ivis 0 relaxation -coll P_ij (sources.f90:37-43) and the body force,
    // projected as the same linear map of the coefficients
    static_assert(src_gram_is_identity<TB>(), "source projection of a linear field is not the identity");
    const T mc = ph.ivis == 0 ? PHC(T, ph, coll) : T(0), bf = PHC(T, ph, body_force);
    sfor<NQ>([&](auto vv) { sfor<NB>([&](auto bb) {
        constexpr int v = decltype(vv)::value, b = decltype(bb)::value;
        T r = rs[(v * NB + b) * TILE_NT + tid];
        if constexpr (v >= PXX) r = fma(mc, q[v][b], r);
        if constexpr (v == MX) r = fma(-bf, q[RH][b], r);
        if constexpr (v == EN) r = fma(-bf, q[MX][b], r);
        rs[(v * NB + b) * TILE_NT + tid] = r;
    }); });
    T* ob = out + B.q0;
    if (a.mode == MODE_RHS) {
        sfor<NQ>([&](auto vv) { sfor<NB>([&](auto bb) {
            constexpr int v = decltype(vv)::value, b = decltype(bb)::value;
            ob[(long long)(b * NQ + v) * nc + le] = rs[(v * NB + b) * TILE_NT + tid];
        }); });
        return;
    }
    const T dt = T(a.st[bx].dt), faci = T(1) / (T(1) + dt * PHC(T, ph, coll));
    const T* q0b = Q0 ? Q0 + B.q0 : nullptr;
    bool bad = false;
    // one variable at a time: the stress rows are stored as they are made;
    // rh..en stay in registers for the next stage's limiter
    auto update = [&](auto vv) {
        constexpr int v = decltype(vv)::value;
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const T r = rs[(v * NB + b) * TILE_NT + tid];              // glflux - source
            T e = q[v][b] - dt * r;                                   // integrator.f90:147-149,171-173
            if (v >= PXX && ph.ivis == 1) e = faci * e;               // :174
            if (a.comb != COMB_NONE) e = rk_combine(a.comb, q0b[(long long)(b * NQ + v) * nc + le], e);
            if (b == 0 && e != e) bad = true;
            if constexpr (v >= PXX) ob[(long long)(b * NQ + v) * nc + le] = e;
            else q[v][b] = e;
        });
    };
    sfor_seq<6>([&](auto mm) { update(std::integral_constant<int, PXX + decltype(mm)::value>{}); });
    sfor_seq<5>([&](auto vv) { update(vv); });
    if (bad) a.flags[0] |= FLAG_NONFINITE;   // integrator.f90:234-250 (the reference exits)
    if (ta.limit_out && (ph.ieos == 1 || ph.ieos == 2)) limit_rows<T, TB>(ph, q);
    sfor<5>([&](auto vv) { sfor<NB>([&](auto bb) {
        constexpr int v = decltype(vv)::value, b = decltype(bb)::value;
        ob[(long long)(b * NQ + v) * nc + le] = q[v][b];
    }); });
}

// k_mindt_limit: hermeshd.f90:145-199 get_min_dt over the cell averages (as
// k_mindt), then, for the step's first stage, the positivity limiter of the
// stage input in place (as k_limit): the time step sees the unlimited state,
// as the reference's step computes dt before euler_step limits Q.
template <class T, class TB>
__global__ void __launch_bounds__(DT_TPB) k_mindt_limit(T* __restrict__ Q, DtArgs a) {
    pdl_enter();
    constexpr int NB = TB::NB;
    const long long gc = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = gc < a.G.ncell;
    int bx = 0;
    double vmag0 = 0.0;
    T q[5][NB];
    long long le = 0, nc = 1;
    T* Qb = Q;
    if (act) {
        bx = box_of_cell(a.G, gc);
        const Box& B = a.G.boxes[bx];
        le = gc - B.cell0;
        nc = B.ncell;
        Qb = Q + B.q0;
        sfor<5>([&](auto vv) { sfor<NB>([&](auto bb) {
            constexpr int v = decltype(vv)::value, b = decltype(bb)::value;
            q[v][b] = Qb[(long long)(b * NQ + v) * nc + le];
        }); });
        const double dn = (double)q[RH][0], dni = 1.0 / dn;
        const double vx = (double)q[MX][0] * dni, vy = (double)q[MY][0] * dni, vz = (double)q[MZ][0] * dni;
        double cs;
        if (a.ph.ieos == 1) cs = sqrt(a.ph.aindex * ((double)q[EN][0] * dni - 0.5 * (vx * vx + vy * vy + vz * vz)));
        else cs = sqrt(7.2 * a.ph.P_1 * pow(dn, 6.2) + a.ph.T_floor);
        const double v0 = fmax(fmax(fabs(vx) + cs, fabs(vy) + cs), fabs(vz) + cs);
        if (v0 > 0.0 && dn > a.ph.rh_mult * a.ph.rh_floor) vmag0 = v0;
        if (le == nc - 1) a.st[bx].cs_last = cs;
    }
    const unsigned full = 0xffffffffu;
    const int bx0 = __shfl_sync(full, bx, 0);
    const bool same = __all_sync(full, bx == bx0 || !act);
    if (same) {
        for (int s = 16; s > 0; s >>= 1) vmag0 = fmax(vmag0, __shfl_xor_sync(full, vmag0, s));
        if ((threadIdx.x & 31) == 0 && vmag0 > 0.0) atomicMax(&a.st[bx0].vmag_bits, (unsigned long long)__double_as_longlong(vmag0));
    } else if (act && vmag0 > 0.0) {
        atomicMax(&a.st[bx].vmag_bits, (unsigned long long)__double_as_longlong(vmag0));
    }
    if (!act || !(a.ph.ieos == 1 || a.ph.ieos == 2)) return;
    // the limiter (k_limit's operations)
    if (q[RH][0] >= PHC(T, a.ph, rh_floor) && limit_bound_clear<TB, T>(a.ph, q)) return;
    bool changed;
    if constexpr (std::is_same<T, double>::value) {
        changed = limit_cell<TB, double>(a.ph, q);
    } else {
        double qd[5][NB];
        sfor<5>([&](auto vv) { sfor<NB>([&](auto bb) { qd[decltype(vv)::value][decltype(bb)::value] = (double)q[decltype(vv)::value][decltype(bb)::value]; }); });
        changed = limit_cell<TB, double>(a.ph, qd);
        sfor<5>([&](auto vv) { sfor<NB>([&](auto bb) { q[decltype(vv)::value][decltype(bb)::value] = (T)qd[decltype(vv)::value][decltype(bb)::value]; }); });
    }
    if (!changed) return;
    sfor<5>([&](auto vv) { sfor<NB>([&](auto bb) {
        constexpr int v = decltype(vv)::value, b = decltype(bb)::value;
        Qb[(long long)(b * NQ + v) * nc + le] = q[v][b];
    }); });
}

}  // namespace hermes

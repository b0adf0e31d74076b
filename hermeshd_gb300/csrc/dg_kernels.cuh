// dg_kernels.cuh -- the CUDA kernels of one SSP-RK stage of the HERMESHD DG
// step, templated on the arithmetic type T and the basis (NB, NQD):
//
//   k_limit  positivity limiter, in place on the stage input (flux.f90:1077-1164)
//   k_face   traces (evaluated here, or read from k_trace's buffer,
//            dg_trace.cuh) + point fluxes + central/LLF + HLLC at every face
//            point of one direction (flux.f90:197-450,466-647; boundary ghosts
//            of prepare_step.f90:20-179 and boundary.f90:40-338 synthesised in place)
//   k_cell   volume quadrature + surface assembly + sources + forward-Euler
//            update + RK combination (flux.f90:751-1022, sources.f90:12-84,
//            integrator.f90:62-252), one write of the stage output; or, split
//            (ivis 0/1, no stochastic stress), the volume quadrature only, with
//   k_update the surface assembly, update and RK combination at one thread
//            per (cell, variable)
//   k_mindt  CFL time step (hermeshd.f90:145-199), FP64 in every precision
//
// Basis and quadrature tables are compile-time constants (dg_tables_gen.cuh)
// and every zero entry is skipped at compile time: on GB300 the FP64 pipe is
// the binding resource of the FP64 path, so each skipped term is time saved.
// For the same reason the kernels use the tables' mirror symmetries (each
// entry at a mirrored point is +- the entry at the point, asserted at compile
// time): values at a mirror pair of points from one even and one odd sum, and
// quadrature sums over a pair as one product with a sum or difference.
#pragma once

#include <cfloat>

#include "dg_physics.cuh"

namespace hermes {

constexpr int LIMIT_TPB = 128;
constexpr int FACE_TPB = 128;
constexpr int CELL_CPB = 32;   // cells per block of k_cell (two threads per cell)
constexpr int DT_TPB = 256;

// stage combination of integrator.f90:62-86
enum Comb { COMB_NONE = 0, COMB_HALF = 1, COMB_34 = 2, COMB_13 = 3 };
enum CellMode { MODE_RHS = 0, MODE_STAGE = 1 };

struct Geom {
    const Box* boxes;
    int nbox;
    int pdl;                  // launch the step kernels with programmatic dependent launch
    long long ncell;          // all boxes
    long long nface[3];       // all boxes, per direction
    long long face0_dir[3];   // faces of the directions before this one (staged face-noise layout)
    // box of each chunk of 32 cells / faces of a direction (ensembles; null
    // for one box): one load instead of a binary search over the boxes
    const int* cbox;
    const int* fbox[3];
};

// the box of global cell gc / face gf of direction DIR: the box of its
// 32-element chunk's first element, stepped over boxes smaller than a chunk
__device__ __forceinline__ int box_of_cell(const Geom& G, long long gc) {
    if (!G.cbox) return find_box(G.boxes, G.nbox, gc, [](const Box& b) { return b.cell0; });
    int bx = __ldg(G.cbox + (gc >> 5));
    while (bx + 1 < G.nbox && G.boxes[bx + 1].cell0 <= gc) ++bx;
    return bx;
}
template <int DIR>
__device__ __forceinline__ int box_of_face(const Geom& G, long long gf) {
    if (!G.fbox[DIR]) return find_box(G.boxes, G.nbox, gf, [](const Box& b) { return b.face0[DIR]; });
    int bx = __ldg(G.fbox[DIR] + (gf >> 5));
    while (bx + 1 < G.nbox && G.boxes[bx + 1].face0[DIR] <= gf) ++bx;
    return bx;
}

// face tables of one direction and side (0 = minus face, 1 = plus face)
template <class TB, int DIR, int SIDE>
__host__ __device__ constexpr double ftab(int p, int b) {
    if constexpr (DIR == 0) return SIDE ? TB::XP(p, b) : TB::XM(p, b);
    else if constexpr (DIR == 1) return SIDE ? TB::YP(p, b) : TB::YM(p, b);
    else return SIDE ? TB::ZP(p, b) : TB::ZM(p, b);
}
template <class TB, int DIR, int SIDE>
__host__ __device__ constexpr double stab(int p, int b) {
    if constexpr (DIR == 0) return SIDE ? TB::SXP(p, b) : TB::SXM(p, b);
    else if constexpr (DIR == 1) return SIDE ? TB::SYP(p, b) : TB::SYM(p, b);
    else return SIDE ? TB::SZP(p, b) : TB::SZM(p, b);
}
template <class TB, int DIR>
__host__ __device__ constexpr double vtab(int g, int b) {
    if constexpr (DIR == 0) return TB::VX(g, b);
    else if constexpr (DIR == 1) return TB::VY(g, b);
    else return TB::VZ(g, b);
}

// Face points in tangential mirror pairs: face point p = i*NE + m, the
// mirror of m is NE-1-m.  Chunk c of a face is a pair (pA = i*NE + NE-1-mc,
// pB = i*NE + mc) or, for an odd point count, the single middle point.
template <class TB>
struct FOrbit {
    static constexpr int NE = TB::NQD, NPAIR = NE / 2, NMC = NPAIR + (NE & 1);
    static constexpr int NCH = NMC * NE;
    static constexpr bool pair(int c) { return c % NMC < NPAIR; }
    static constexpr int pA(int c) { return (c / NMC) * NE + (pair(c) ? NE - 1 - c % NMC : NPAIR); }
    static constexpr int pB(int c) { return pair(c) ? (c / NMC) * NE + c % NMC : pA(c); }
};

// the face tables of one direction by side: point values (SURF false) or
// surface quadrature weights (SURF true)
template <class TB, int DIR, bool SURF>
__host__ __device__ constexpr double face_tab(int side, int p, int b) {
    if constexpr (SURF) return side ? stab<TB, DIR, 1>(p, b) : stab<TB, DIR, 0>(p, b);
    else return side ? ftab<TB, DIR, 1>(p, b) : ftab<TB, DIR, 0>(p, b);
}
// parity class of basis function b at chunk c: bit 0 = odd in the normal
// coordinate (the minus-face entry is the negated plus-face entry), bit 1 =
// odd in the tangential mirror; -1 where the entry is zero
template <class TB, int DIR, bool SURF>
__host__ __device__ constexpr int face_class(int c, int b) {
    using FO = FOrbit<TB>;
    const double a = face_tab<TB, DIR, SURF>(1, FO::pA(c), b);
    if (a == 0.0) return -1;
    const double mn = face_tab<TB, DIR, SURF>(0, FO::pA(c), b), tb = face_tab<TB, DIR, SURF>(1, FO::pB(c), b);
    return (mn == a ? 0 : 1) | (tb == a ? 0 : 2);
}
// every entry of the four (side, point) combinations of a chunk is +-the
// (plus, pA) entry, the (minus, pB) sign being the product of the other two
template <class TB, int DIR, bool SURF>
__host__ __device__ constexpr bool face_tables_symmetric() {
    using FO = FOrbit<TB>;
    for (int c = 0; c < FO::NCH; ++c)
        for (int b = 0; b < TB::NB; ++b) {
            const double a = face_tab<TB, DIR, SURF>(1, FO::pA(c), b);
            const double mn = face_tab<TB, DIR, SURF>(0, FO::pA(c), b), tb = face_tab<TB, DIR, SURF>(1, FO::pB(c), b);
            const double mb = face_tab<TB, DIR, SURF>(0, FO::pB(c), b);
            if (mn != a && mn != -a) return false;
            if (tb != a && tb != -a) return false;
            const double sn = mn == a ? 1.0 : -1.0, st = tb == a ? 1.0 : -1.0;
            if (mb != sn * st * a) return false;
            if (!FO::pair(c) && tb != a) return false;
        }
    return true;
}
template <class TB, int DIR, bool SURF>
__host__ __device__ constexpr bool face_has(int c, int k) {
    for (int b = 0; b < TB::NB; ++b)
        if (face_class<TB, DIR, SURF>(c, b) == k) return true;
    return false;
}

// a + b and a - b where a or b may be an empty (compile-time zero) sum
template <bool HA, bool HB, class T>
__device__ __forceinline__ T sum_opt(T a, T b) {
    if constexpr (HA && HB) return a + b;
    else if constexpr (HA) return a;
    else if constexpr (HB) return b;
    else return T(0);
}
template <bool HA, bool HB, class T>
__device__ __forceinline__ T diff_opt(T a, T b) {
    if constexpr (HA && HB) return a - b;
    else if constexpr (HA) return a;
    else if constexpr (HB) return -b;
    else return T(0);
}

// trace of all NQ variables of one cell at face point P: sum_b phi_b(P) Q(b,v)
template <class TB, int DIR, int SIDE, int P, class T>
__device__ __forceinline__ void trace_pt(const T* __restrict__ Qb, long long ncell, long long cell, T out[NQ]) {
    sfor<NQ>([&](auto vv) {
        constexpr int v = decltype(vv)::value;
        T acc = T(0);
        sfor<TB::NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            constexpr double c = ftab<TB, DIR, SIDE>(P, b);
            if constexpr (c != 0.0) acc = fma(T(c), __ldg(Qb + (long long)(b * NQ + v) * ncell + cell), acc);
        });
        out[v] = acc;
    });
}

// trace of a single variable at face point P
template <class TB, int DIR, int SIDE, int P, int V, class T>
__device__ __forceinline__ T trace_var(const T* __restrict__ Qb, long long ncell, long long cell) {
    T acc = T(0);
    sfor<TB::NB>([&](auto bb) {
        constexpr int b = decltype(bb)::value;
        constexpr double c = ftab<TB, DIR, SIDE>(P, b);
        if constexpr (c != 0.0) acc = fma(T(c), __ldg(Qb + (long long)(b * NQ + V) * ncell + cell), acc);
    });
    return acc;
}

// ===========================================================================
// k_limit: flux.f90:1077-1164, in place.  One thread per cell.
// Fast path: a bound on every face-point value, |sum_{b>0} phi_b q_b| <=
// sum_{b>0} max_p|phi_b(p)| |q_b|, proves that no point can trigger the
// density or pressure branch; the cell is then left untouched, which is what
// the full evaluation would do.  Only cells the bound cannot clear run the
// point-by-point evaluation.  For T = float the evaluation near the floors
// runs in FP64.
// ===========================================================================
template <class TB>
__host__ __device__ constexpr double lim_maxabs(int b) {
    double m = 0.0;
    for (int p = 0; p < TB::NPGE; ++p) {
        double a = TB::LIM(p, b) < 0 ? -TB::LIM(p, b) : TB::LIM(p, b);
        if (a > m) m = a;
    }
    return m;
}

// the rh..en rows of one cell held elsewhere than a register array: element
// (v, b) at p[v * row + b * col] (shared memory in k_update)
template <class T>
struct StridedRows {
    T* p;
    int row, col;
    struct Row {
        T* p;
        int col;
        __device__ __forceinline__ T& operator[](int b) const { return p[b * col]; }
    };
    __device__ __forceinline__ Row operator[](int v) const { return Row{p + v * row, col}; }
};

// q: the rh..en rows, q[v][b] (a U[5][NB] register array or StridedRows<U>)
template <class TB, class U, class QA>
__device__ __forceinline__ bool limit_cell(const Phys& ph, QA& q) {
    // returns true if q was modified
    constexpr int NB = TB::NB;
    const U rh_floor = PHC(U, ph, rh_floor), epsi = PHC(U, ph, rh_floor), epsiP = PHC(U, ph, rh_floor) * PHC(U, ph, T_floor);
    const U aindm1 = PHC(U, ph, aindm1);
    if (q[RH][0] < rh_floor) {
        sfor<NB - 1>([&](auto bb) {
            constexpr int b = decltype(bb)::value + 1;
            q[RH][b] = U(0); q[MX][b] = U(0); q[MY][b] = U(0); q[MZ][b] = U(0); q[EN][b] = U(0);
        });
        q[RH][0] = rh_floor;
        return true;
    }
    bool changed = false;
    // density at the npge face points
    U Qrhmin = U(0);
    sfor<TB::NPGE>([&](auto pp) {
        constexpr int p = decltype(pp)::value;
        U s = U(0);
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            constexpr double c = TB::LIM(p, b);
            if constexpr (c != 0.0) s = fma(U(c), q[RH][b], s);
        });
        if (p == 0 || s < Qrhmin) Qrhmin = s;
    });
    if (Qrhmin < epsi) {
        U theta = (epsi - q[RH][0]) / (Qrhmin - q[RH][0]);
        if (theta > U(1)) theta = U(1);
        if (theta < U(0)) theta = U(0);
        sfor<NB - 1>([&](auto bb) {
            constexpr int b = decltype(bb)::value + 1;
            q[RH][b] = fabs(theta) * q[RH][b];
        });
        changed = true;
    }
    const U Pave = aindm1 * (q[EN][0] - U(0.5) * (q[MX][0] * q[MX][0] + q[MY][0] * q[MY][0] + q[MZ][0] * q[MZ][0]) / q[RH][0]);
    if (Pave < epsiP) {
        sfor<NB - 1>([&](auto bb) {
            constexpr int b = decltype(bb)::value + 1;
            q[RH][b] = U(0); q[MX][b] = U(0); q[MY][b] = U(0); q[MZ][b] = U(0); q[EN][b] = U(0);
        });
        return true;
    }
    U theta = U(1);
    sfor<TB::NPGE>([&](auto pp) {
        constexpr int p = decltype(pp)::value;
        U e[5];
        sfor<5>([&](auto vv) {
            constexpr int v = decltype(vv)::value;
            U s = U(0);
            sfor<NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                constexpr double c = TB::LIM(p, b);
                if constexpr (c != 0.0) s = fma(U(c), q[v][b], s);
            });
            e[v] = s;
        });
        U dni = U(1) / e[RH];
        U P = aindm1 * (e[EN] - U(0.5) * dni * (e[MX] * e[MX] + e[MY] * e[MY] + e[MZ] * e[MZ]));
        if (P < epsiP) {
            if (Pave != P) theta = fmin(theta, (Pave - epsiP) / (Pave - P));
        }
    });
    if (theta > U(1)) theta = U(1);
    if (theta < U(0)) theta = U(0);
    if (theta != U(1)) {
        sfor<NB - 1>([&](auto bb) {
            constexpr int b = decltype(bb)::value + 1;
            sfor<5>([&](auto vv) { q[decltype(vv)::value][b] = theta * q[decltype(vv)::value][b]; });
        });
        changed = true;
    }
    return changed;
}

template <class TB, class U, class QA>
__device__ __forceinline__ bool limit_bound_clear(const Phys& ph, const QA& q) {
    // true if no face point can fall below the density or pressure floor
    constexpr int NB = TB::NB;
    U B[5];
    sfor<5>([&](auto vv) {
        constexpr int v = decltype(vv)::value;
        U s = U(0);
        sfor<NB - 1>([&](auto bb) {
            constexpr int b = decltype(bb)::value + 1;
            constexpr double m = lim_maxabs<TB>(b);
            if constexpr (m != 0.0) s = fma(U(m), fabs(q[v][b]), s);
        });
        B[v] = s;
    });
    const U tol = U(std::is_same<U, double>::value ? 1e-10 : 1e-4);
    const U epsi = PHC(U, ph, rh_floor), epsiP = PHC(U, ph, rh_floor) * PHC(U, ph, T_floor);
    U rlo = q[RH][0] - B[RH];
    if (!(rlo >= epsi + tol * (q[RH][0] + B[RH]))) return false;
    U Elo = q[EN][0] - B[EN];
    U m0 = fabs(q[MX][0]) + B[MX], m1 = fabs(q[MY][0]) + B[MY], m2 = fabs(q[MZ][0]) + B[MZ];
    U ke = U(0.5) * (m0 * m0 + m1 * m1 + m2 * m2) / rlo;
    U Plo = PHC(U, ph, aindm1) * (Elo - ke);
    return Plo >= epsiP + tol * (fabs(q[EN][0]) + B[EN] + ke);
}

template <class T, class TB>
__global__ void __launch_bounds__(LIMIT_TPB) k_limit(T* __restrict__ Q, Geom G, Phys ph) {
    pdl_enter();
    constexpr int NB = TB::NB;
    long long gc = (long long)blockIdx.x * LIMIT_TPB + threadIdx.x;
    if (gc >= G.ncell) return;
    int bx = box_of_cell(G, gc);
    const Box& B = G.boxes[bx];
    const long long le = gc - B.cell0, nc = B.ncell;
    T* Qb = Q + B.q0;
    T q[5][NB];
    sfor<5>([&](auto vv) {
        constexpr int v = decltype(vv)::value;
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            q[v][b] = Qb[(long long)(b * NQ + v) * nc + le];
        });
    });
    if (q[RH][0] >= PHC(T, ph, rh_floor) && limit_bound_clear<TB, T>(ph, q)) return;
    bool changed;
    if constexpr (std::is_same<T, double>::value) {
        changed = limit_cell<TB, double>(ph, q);
    } else {
        // FP64 positivity fix for the FP32 path
        double qd[5][NB];
        sfor<5>([&](auto vv) { sfor<NB>([&](auto bb) { qd[decltype(vv)::value][decltype(bb)::value] = (double)q[decltype(vv)::value][decltype(bb)::value]; }); });
        changed = limit_cell<TB, double>(ph, qd);
        sfor<5>([&](auto vv) { sfor<NB>([&](auto bb) { q[decltype(vv)::value][decltype(bb)::value] = (T)qd[decltype(vv)::value][decltype(bb)::value]; }); });
    }
    if (!changed) return;
    sfor<5>([&](auto vv) {
        constexpr int v = decltype(vv)::value;
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            Qb[(long long)(b * NQ + v) * nc + le] = q[v][b];
        });
    });
}

// ===========================================================================
// k_face: one thread per (face, point).  blockIdx.y = face point P.
// ===========================================================================
struct FaceArgs {
    Geom G;
    Phys ph;
    const unsigned long long* step;  // noise step counter (device)
    unsigned stage;
    int tpb;                         // faces per block (32, 64 or 128; 0 = FACE_TPB)
    const void* noise;               // staged stochastic stress of the faces (k_noise_face), or null: drawn here
    const void* traces;              // face traces of every cell (k_trace), or null: evaluated here
    int point_loop;                  // one thread per face looping over its points (k_face_pl)
};

// where k_face takes the traces of its two cells from: evaluated from the
// coefficients (TRB false) or read from the buffer k_trace wrote, laid out
// [direction][side][variable][point][cell of the whole grid]
template <class T, class TB, int DIR, bool TRB>
struct FaceTraces {
    const T* Qb;          // coefficients of the box
    long long nc;         // cells of the box
    const T* tr;          // trace buffer
    long long ncl;        // cells of the grid
    long long cell0;      // first cell of the box
    template <int SIDE>
    __device__ __forceinline__ const T* slot(long long c) const {
        return tr + (long long)((DIR * 2 + SIDE) * NQ) * TB::NF * ncl + cell0 + c;
    }
    template <int SIDE, int P>
    __device__ __forceinline__ void pt(long long c, T q[NQ]) const {
        if constexpr (TRB) {
            const T* t = slot<SIDE>(c) + (long long)P * ncl;
#pragma unroll
            for (int v = 0; v < NQ; ++v) q[v] = __ldg(t + (long long)v * TB::NF * ncl);
        } else {
            trace_pt<TB, DIR, SIDE, P>(Qb, nc, c, q);
        }
    }
    template <int SIDE, int P, int V>
    __device__ __forceinline__ T var(long long c) const {
        if constexpr (TRB) return __ldg(slot<SIDE>(c) + (long long)(V * TB::NF + P) * ncl);
        else return trace_var<TB, DIR, SIDE, P, V>(Qb, nc, c);
    }
};

// the numerical flux at one face point from the two traces (after boundary
// ghosts): point fluxes of both sides (flux.f90:240), central flux or LLF
// with the freezing speed (flux.f90:243-262), then HLLC (flux.f90:264-271) or
// Roe (SEAN monolith) for rh..en.  Shared by k_face and the adjoint.
// F comes out multiplied by sc (the face kernel's inverse spacing): the
// central rows as (fL + fR) * (0.5 sc), the same rounding as 0.5 (fL + fR)
// scaled afterwards, since 0.5 sc is exact; with HLLC the central values of
// rh..en, which HLLC replaces, are not formed.
template <class T, int DIR>
__device__ __forceinline__ void face_flux_fn(const Phys& ph, const T qL[NQ], const T qR[NQ], const T SL[6], const T SR[6],
                                             T rho_i_last, T F[NQ], T sc = T(1)) {
    T fL[NQ], fR[NQ];
    const Prim<T> wL = primitives(ph, qL);
    point_flux<T, DIR>(ph, qL, wL, SL, fL);
    const Prim<T> wR = primitives(ph, qR);
    point_flux<T, DIR>(ph, qR, wR, SR, fR);
    if (ph.ivis >= 2) {   // ivis 3: the Grad-closure code always applies LLF (ten_moment.f90:1131-1147)
        const T cfr = fmax(cfcal<T, DIR>(ph, qL), cfcal<T, DIR>(ph, qR));
#pragma unroll
        for (int v = 0; v < NQ; ++v) F[v] = (T(0.5) * (fL[v] + fR[v]) - T(0.5) * cfr * (qR[v] - qL[v])) * sc;
    } else {
        const T h = T(0.5) * sc;
        const bool hl = ph.ihllc == 1;
#pragma unroll
        for (int v = 0; v < NQ; ++v)
            if (v >= PXX || !hl) F[v] = (fL[v] + fR[v]) * h;
    }
    if (ph.ihllc == 2) {
        T FR[NQ];
        if (roe<T, DIR>(ph, qL, qR, fL, fR, FR)) {
            F[RH] = FR[RH] * sc; F[MX] = FR[MX] * sc; F[MY] = FR[MY] * sc; F[MZ] = FR[MZ] * sc; F[EN] = FR[EN] * sc;
        }
    } else if (ph.ihllc == 1) {
        hllc<T, DIR>(ph, qL, qR, fL, fR, wL, wR, rho_i_last, F);
#pragma unroll
        for (int v = RH; v <= EN; ++v) F[v] = F[v] * sc;
    }
}

template <class T, class TB, int DIR, int P, bool NOISE, bool TRB>
__device__ __forceinline__ void face_point(const T* __restrict__ Q, T* __restrict__ flux, const FaceArgs& a, long long gf) {
    const Geom& G = a.G;
    const Phys& ph = a.ph;
    int bx = box_of_face<DIR>(G, gf);
    const Box& B = G.boxes[bx];
    const long long lf = gf - B.face0[DIR];
    const int n0 = B.n[0], n1 = B.n[1], n2 = B.n[2];
    const int ex = DIR == 0 ? B.nfp[0] : n0, ey = DIR == 1 ? B.nfp[1] : n1;
    // 32-bit division (a box has fewer than 2^31 faces per direction, checked
    // at context creation): a 64-bit division costs as much as an FP32 face
    const unsigned lfu = (unsigned)lf, t = lfu / (unsigned)ex;
    const int i = (int)(lfu - t * (unsigned)ex);
    const int j = (int)(t % (unsigned)ey);
    const int k = (int)(t / (unsigned)ey);
    const int n = B.n[DIR];
    const int s = DIR == 0 ? i : DIR == 1 ? j : k;       // face plane
    const bool dedup = B.nfp[DIR] == n;                    // both ends periodic: n planes
    const long long nc = B.ncell;
    const FaceTraces<T, TB, DIR, TRB> ts{Q + B.q0, nc, static_cast<const T*>(a.traces), G.ncell, B.cell0};
    auto cell_at = [&](int c) -> long long {              // cell with plane coordinate c
        int ci = DIR == 0 ? c : i, cj = DIR == 1 ? c : j, ck = DIR == 2 ? c : k;
        return (long long)ci + (long long)n0 * (cj + (long long)n1 * ck);
    };
    constexpr int MN = DIR == 0 ? MX : DIR == 1 ? MY : MZ;   // normal momentum
    T qL[NQ], qR[NQ];
    if (dedup || (s > 0 && s < n)) {
        const int lo = s > 0 ? s - 1 : n - 1;
        ts.template pt<1, P>(cell_at(lo), qL);
        ts.template pt<0, P>(cell_at(s), qR);
    } else if (s == 0) {
        // low boundary: ghost from the first cell's minus trace (boundary.f90:40-244)
        const long long c0 = cell_at(0);
        ts.template pt<0, P>(c0, qR);
        const int code = B.bc[2 * DIR];
        if (code == BC_PERIODIC) {
            // topology not periodic (the hi flag is not): the ghost is the never-received zero trace
            for (int v = 0; v < NQ; ++v) qL[v] = T(0);
        } else {
            for (int v = 0; v < NQ; ++v) qL[v] = qR[v];
            if (DIR == 0 && code == BC_INFLOW) {
                // boundary.f90:568-612: rho, m_x, E of the parabolic profile at the
                // face row's cell centre yc(j); m_y = m_z = 0; the stresses copied
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
                sfor<TB::NF>([&](auto pp) {
                    mmax = fmax(mmax, ts.template var<0, decltype(pp)::value, MN>(c0));
                });
                if (mmax > T(0)) qL[MN] = T(0);
            }
        }
    } else {
        // high boundary (s == n)
        const long long cl = cell_at(n - 1);
        ts.template pt<1, P>(cl, qL);
        const int code = B.bc[2 * DIR + 1];
        if (code == BC_PERIODIC) {
            // periodic topology with a non-periodic low flag: the ghost is the
            // first cell's raw minus trace (prepare_step.f90:75-104 self-send)
            ts.template pt<0, P>(cell_at(0), qR);
        } else if (code == BC_OUTFLOW && DIR == 0) {
            // boundary.f90:246-282 never copies the interior trace: from a zero
            // ghost array the result stays zero
            for (int v = 0; v < NQ; ++v) qR[v] = T(0);
        } else {
            for (int v = 0; v < NQ; ++v) qR[v] = qL[v];
            if (code == BC_NOSLIP) { qR[MX] = T(0); qR[MY] = T(0); qR[MZ] = T(0); }
            else if (code == BC_WALL) { qR[MN] = T(0); }
            else if (code == BC_OUTFLOW) {
                T mmin = T(INFINITY);
                sfor<TB::NF>([&](auto pp) {
                    mmin = fmin(mmin, ts.template var<1, decltype(pp)::value, MN>(cl));
                });
                if (mmin < T(0)) qR[MN] = T(0);
            }
        }
    }
    // point fluxes of both sides (flux.f90:240), stochastic stress per side
    T SL[6] = {T(0), T(0), T(0), T(0), T(0), T(0)}, SR[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
    if constexpr (NOISE) {
        if (a.noise) {
            // [side][component][point][face] of this direction (dg_noise.cuh)
            const T* nb = static_cast<const T*>(a.noise) + 12ll * TB::NF * G.face0_dir[DIR];
            const long long nfa = G.nface[DIR];
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                SL[c] = nb[((long long)(0 * 6 + c) * TB::NF + P) * nfa + gf];
                SR[c] = nb[((long long)(1 * 6 + c) * TB::NF + P) * nfa + gf];
            }
        } else {
            NoiseCtr nc_{*a.step, a.stage};
            random_stress<T>(ph, B.seed, nc_, DIR, (unsigned long long)lf, P, SL);
            random_stress<T>(ph, B.seed, nc_, DIR, (unsigned long long)lf, P + TB::NF, SR);
        }
    }
    T F[NQ];
    T rho_i_last = T(0);
    if (ph.ihllc == 1) {
        if (ph.ieos == 2) {
            // 1/rho of the last point of the reference's call: the right state at point NF-1
            T rlast;
            if (dedup || s < n) rlast = ts.template var<0, TB::NF - 1, RH>(cell_at(s));
            else if (B.bc[2 * DIR + 1] == BC_PERIODIC) rlast = ts.template var<0, TB::NF - 1, RH>(cell_at(0));
            else if (B.bc[2 * DIR + 1] == BC_OUTFLOW && DIR == 0) rlast = T(0);
            else rlast = ts.template var<1, TB::NF - 1, RH>(cell_at(n - 1));
            rho_i_last = T(1) / rlast;
        }
    }
    // scaled by the inverse spacing of this direction
    face_flux_fn<T, DIR>(ph, qL, qR, SL, SR, rho_i_last, F, T(B.di[DIR]));
    const long long nfd = (long long)ex * ey * (DIR == 2 ? B.nfp[2] : n2);
    T* fb = flux + B.fbase[DIR];
#pragma unroll
    for (int v = 0; v < NQ; ++v) fb[(long long)(v * TB::NF + P) * nfd + lf] = F[v];
}

// resident blocks per SM the face kernel's register allocation must allow:
// FP64 is FP64-pipe bound at 4 (128 registers); FP32 has the arithmetic to
// spare and gains from more resident warps (6 blocks: 80 registers)
template <class T>
struct FaceMinBlocks {
    static constexpr int value = std::is_same<T, float>::value ? 6 : 4;
};

template <class T, class TB, int DIR, bool NOISE, bool TRB>
__global__ void __launch_bounds__(FACE_TPB, (FaceMinBlocks<T>::value)) k_face(const T* __restrict__ Q, T* __restrict__ flux, FaceArgs a) {
    pdl_enter();
    long long gf = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gf >= a.G.nface[DIR]) return;
    const int p = blockIdx.y;
    sfor<TB::NF>([&](auto pp) {
        constexpr int P = decltype(pp)::value;
        if (p == P) face_point<T, TB, DIR, P, NOISE, TRB>(Q, flux, a, gf);
    });
}

// the faces of all three directions in one launch: blockIdx.z = direction,
// blockIdx.y = face point (the blocks of a direction with fewer faces than
// the largest return at once).  One launch instead of three per stage lets
// the directions fill each other's tails.
template <class T, class TB, bool NOISE, bool TRB>
__global__ void __launch_bounds__(FACE_TPB, (FaceMinBlocks<T>::value)) k_faces(const T* __restrict__ Q, T* __restrict__ flux, FaceArgs a) {
    pdl_enter();
    const long long gf = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int dir = blockIdx.z, p = blockIdx.y;
    if (gf >= a.G.nface[dir]) return;
    sfor<3>([&](auto dd) {
        constexpr int D = decltype(dd)::value;
        if (dir == D) {
            sfor<TB::NF>([&](auto pp) {
                constexpr int P = decltype(pp)::value;
                if (p == P) face_point<T, TB, D, P, NOISE, TRB>(Q, flux, a, gf);
            });
        }
    });
}

// ===========================================================================
// k_cell: two threads per cell.  In a block of 2*CELL_CPB threads, thread
// c < CELL_CPB owns the hydro variables rh..en of cell c and thread
// CELL_CPB + c owns the six stress variables of the same cell (each group
// fills whole warps).  The cell's coefficients are shared through one
// shared-memory column per cell; each thread evaluates its own variables at
// the quadrature points and the pair swaps them through an exchange buffer,
// one x-mirror orbit of points at a time; each thread keeps the
// volume-quadrature accumulators of its own variables in registers.
// ===========================================================================
struct CellArgs {
    Geom G;
    Phys ph;
    const BoxState* st;               // dt per box
    const unsigned long long* step;   // noise step counter
    int* flags;
    unsigned stage;
    int mode, comb;
    int split_source;   // Grad closure with RK2: the implicit source step after the update
    const void* noise;  // staged interior stochastic stress (k_noise_cell), or null: drawn here
    void* accbuf;       // split update: k_cell stores the volume terms here, k_update finishes
    int limit_out;      // k_update (FP64): apply the next stage's positivity limiter to the output
    int utpb = 0;       // threads per block of k_update (0: UPD_TPB)
    int phase = 0;      // split update: 0 both kernels, 1 the volume kernel only, 2 the update only
};

// RK combination of integrator.f90:62-86
template <class T>
__device__ __forceinline__ T rk_combine(int comb, T q0, T e) {
    if (comb == COMB_HALF) return T(0.5) * (q0 + e);                         // integrator.f90:70
    if (comb == COMB_34) return T(0.75) * q0 + T(0.25) * e;                  // integrator.f90:82
    return T(1.0 / 3.0) * q0 + T(2.0 / 3.0) * e;                            // integrator.f90:85
}

// what the phases of one cell share
template <class T>
struct CellCtx {
    const T* qs_base;
    T* qs;            // shared column base of this block
    T* ub;            // exchange buffer of the point values, [2][NQ][2][CELL_CPB]
    int lc;           // cell slot in the block
    bool act;
    int bx;
    long long le, nc;
    const Box* B;
    T di[3];
    NoiseCtr nctr;
    bool noise;
    T dt, faci;
    T* ob;
    const T* q0b;
    long long fm[3], fp[3], nfd[3];
    bool bad;
};

// The interior points in x-mirror orbits: chunk c is the pair gA (x = +xq)
// and gB (x = -xq) with the same (y, z), or, for an odd point count, the one
// point at x = 0.  Every table row of gB is the row of gA with the sign of
// the basis function's parity in x (checked at compile time), so a
// variable's values at the pair are E + O and E - O (E, O: the sums over the
// even and the odd functions at gA), and the pair's contributions to a
// quadrature sum are c (f_A + f_B) or c (f_A - f_B): half the table products.
template <class TB>
struct XOrbit {
    static constexpr int NE = TB::NQD, NE2 = NE * NE, NPAIR = NE / 2;
    static constexpr int NCH = (NPAIR + (NE & 1)) * NE2;
    static constexpr bool pair(int c) { return c / NE2 < NPAIR; }
    static constexpr int gA(int c) { return pair(c) ? (NE - 1 - c / NE2) * NE2 + c % NE2 : NPAIR * NE2 + c % NE2; }
    static constexpr int gB(int c) { return pair(c) ? (c / NE2) * NE2 + c % NE2 : gA(c); }
};

// sum_g SRC(g, b) INT(g, b2): the quadrature of the source projection applied
// to a field that is linear in the state.  The Gauss rules integrate these
// products exactly and the basis is orthogonal with SRC normalised by cbasis,
// so this is the identity to rounding (asserted where it is used): a source
// linear in the state (ivis 0 relaxation -coll P_ij, the body force)
// projects to the same linear map of the coefficients.
template <class TB>
__host__ __device__ constexpr double src_gram(int b, int b2) {
    double s = 0.0;
    for (int g = 0; g < TB::NPG; ++g) s += TB::SRC(g, b) * TB::INT(g, b2);
    return s;
}
template <class TB>
__host__ __device__ constexpr bool src_gram_is_identity() {
    for (int b = 0; b < TB::NB; ++b)
        for (int b2 = 0; b2 < TB::NB; ++b2) {
            const double e = src_gram<TB>(b, b2) - (b == b2 ? 1.0 : 0.0);
            if (e > 1e-14 || e < -1e-14) return false;
        }
    return true;
}

// the values of one thread group's variables at the points of x-orbit chunk
// c, written to the exchange buffer slot ubc ([NQ][2][CELL_CPB])
template <class T, class TB, int GRP, int c>
__device__ __forceinline__ void chunk_eval(const volatile T* qs, volatile T* ubc, int lc) {
    using XO = XOrbit<TB>;
    constexpr int NB = TB::NB;
    constexpr int GV0 = GRP == 0 ? 0 : PXX;
    constexpr int GNV = GRP == 0 ? 5 : 6;
    constexpr bool PAIR = XO::pair(c);
    constexpr int gA = XO::gA(c), gB = XO::gB(c);
    sfor<GNV>([&](auto mm) {
        constexpr int v = GV0 + decltype(mm)::value;
        T E = T(0), O = T(0);
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            constexpr double cA = TB::INT(gA, b), cB = TB::INT(gB, b);
            static_assert(cB == cA || cB == -cA, "interior table not mirror-symmetric in x");
            if constexpr (cA != 0.0) {
                const T q = qs[(b * NQ + v) * CELL_CPB + lc];
                if constexpr (cB == cA) E = fma(T(cA), q, E);
                else O = fma(T(cA), q, O);
            }
        });
        if constexpr (PAIR) {
            ubc[(v * 2 + 0) * CELL_CPB + lc] = E + O;
            ubc[(v * 2 + 1) * CELL_CPB + lc] = E - O;
        } else {
            ubc[(v * 2 + 0) * CELL_CPB + lc] = E;
        }
    });
}

// some point of the volume table of direction d has a nonzero weight for b
template <class TB, int d>
__host__ __device__ constexpr bool vtab_any(int b) {
    for (int g = 0; g < TB::NPG; ++g)
        if (vtab<TB, d>(g, b) != 0.0) return true;
    return false;
}

// phase 1 of the stress group for ivis 0 and 1: the stress fluxes are
// colvis-weighted velocity components (flux.f90:57-62 and the y, z rows),
// f_d[m] = K(d, m) v_j(d, m), so the volume quadrature of all six rows is
// made of the nine sums V[d][j][b] = sum_g vtab_d(g, b) v_j(g), combined with
// the constants once at the end: three products per point and direction
// instead of six, and no per-point flux rows.
template <class T, class TB, bool NOISE>
__device__ __forceinline__ void cell_volume_linear_stress(const CellArgs& a, CellCtx<T>& cx, T (&acc)[6][TB::NB]) {
    using XO = XOrbit<TB>;
    constexpr int NB = TB::NB;
    const Phys& ph = a.ph;
    const volatile T* qs = cx.qs;
    volatile T* ub = cx.ub;
    const int lc = cx.lc;
    const bool act = cx.act;
    T V[3][3][NB];
    sfor<3>([&](auto dd) { sfor<3>([&](auto jj) { sfor<NB>([&](auto bb) {
        V[decltype(dd)::value][decltype(jj)::value][decltype(bb)::value] = T(0); }); }); });
    sfor_seq<XO::NCH>([&](auto cc) {
        constexpr int c = decltype(cc)::value;
        constexpr bool PAIR = XO::pair(c);
        constexpr int gA = XO::gA(c), gB = XO::gB(c);
        constexpr int NK = PAIR ? 2 : 1;
        volatile T* ubc = ub + (c & 1) * (NQ * 2 * CELL_CPB);
        if (act) chunk_eval<T, TB, 1, c>(qs, ubc, lc);
        block_sync_split();
        if (act) {
            T vel[NK][3];
            sfor<NK>([&](auto kk) {
                constexpr int k = decltype(kk)::value;
                const T dni = T(1) / T(ubc[(RH * 2 + k) * CELL_CPB + lc]);
                sfor<3>([&](auto jj) {
                    constexpr int j = decltype(jj)::value;
                    vel[k][j] = T(ubc[((MX + j) * 2 + k) * CELL_CPB + lc]) * dni;
                });
            });
            T vs[3], vd[3];
            sfor<3>([&](auto jj) {
                constexpr int j = decltype(jj)::value;
                if constexpr (PAIR) { vs[j] = vel[0][j] + vel[NK - 1][j]; vd[j] = vel[0][j] - vel[NK - 1][j]; }
                else { vs[j] = vel[0][j]; vd[j] = vel[0][j]; }
            });
            sfor<3>([&](auto dd) {
                constexpr int d = decltype(dd)::value;
                sfor<NB>([&](auto bb) {
                    constexpr int b = decltype(bb)::value;
                    constexpr double cA = vtab<TB, d>(gA, b), cB = vtab<TB, d>(gB, b);
                    static_assert(cB == cA || cB == -cA, "volume table not mirror-symmetric in x");
                    if constexpr (cA != 0.0) {
                        sfor<3>([&](auto jj) {
                            constexpr int j = decltype(jj)::value;
                            V[d][j][b] = fma(T(cA), (!PAIR || cB == cA) ? vs[j] : vd[j], V[d][j][b]);
                        });
                    }
                });
            });
        }
    });
    if (!act) return;
    // K(d, m) di_d: diagonal rows (4/3, -2/3, -2/3) colvis v_d, off-diagonal colvis v_other
    const T cv = PHC(T, ph, colvis), c4 = T(4.0 / 3.0) * cv, c2 = -(T(2.0 / 3.0) * cv);
    sfor<3>([&](auto dd) {
        constexpr int d = decltype(dd)::value;
        const T di = cx.di[d];
        const T kdiag = c4 * di, koff = c2 * di, kcv = cv * di;
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            if constexpr (vtab_any<TB, d>(b)) {
                // rows pxx, pyy, pzz: v_d with 4/3 on the row of d, -2/3 on the others
                sfor<3>([&](auto ii) {
                    constexpr int i = decltype(ii)::value;
                    acc[i][b] = fma(i == d ? kdiag : koff, V[d][d][b], acc[i][b]);
                });
                // pxy (m 3), pxz (m 4), pyz (m 5): colvis times the other index's velocity
                if constexpr (d == 0) {
                    acc[3][b] = fma(kcv, V[0][1][b], acc[3][b]);
                    acc[4][b] = fma(kcv, V[0][2][b], acc[4][b]);
                } else if constexpr (d == 1) {
                    acc[3][b] = fma(kcv, V[1][0][b], acc[3][b]);
                    acc[5][b] = fma(kcv, V[1][2][b], acc[5][b]);
                } else {
                    acc[4][b] = fma(kcv, V[2][0][b], acc[4][b]);
                    acc[5][b] = fma(kcv, V[2][1][b], acc[5][b]);
                }
            }
        });
    });
    if (ph.ivis == 0) {   // sources.f90:37-43, linear: the coefficients themselves (src_gram)
        static_assert(src_gram_is_identity<TB>(), "source projection of a linear field is not the identity");
        const T mc = -PHC(T, ph, coll);
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            sfor<6>([&](auto mm) {
                constexpr int m = decltype(mm)::value;
                acc[m][b] = fma(mc, T(qs[(b * NQ + PXX + m) * CELL_CPB + lc]), acc[m][b]);
            });
        });
    }
}

// phase 1: volume quadrature and point sources of one group's variables
// (flux.f90:751-928, sources.f90:28-78); acc collects volume + source.  Each
// thread evaluates only its own group's variables at the points and the two
// threads of a cell swap them through the exchange buffer (one block barrier
// per orbit; every thread of the block, active or not, runs the same loop).
template <class T, class TB, int GRP, bool NOISE>
__device__ __forceinline__ void cell_volume(const CellArgs& a, CellCtx<T>& cx, T (&acc)[6][TB::NB]) {
    using XO = XOrbit<TB>;
    constexpr int NB = TB::NB, NPG = TB::NPG;
    constexpr int GV0 = GRP == 0 ? 0 : PXX;
    constexpr int GNV = GRP == 0 ? 5 : 6;
    const Phys& ph = a.ph;
    if constexpr (GRP == 1) {
        if (ph.ivis < 2) {   // uniform over the block: both groups run the same number of barriers
            cell_volume_linear_stress<T, TB, NOISE>(a, cx, acc);
            return;
        }
    }
    const volatile T* qs = cx.qs;
    volatile T* ub = cx.ub;   // [2][NQ][2][CELL_CPB]
    const int lc = cx.lc;
    const bool act = cx.act;
    sfor_seq<XO::NCH>([&](auto cc) {
        constexpr int c = decltype(cc)::value;
        constexpr bool PAIR = XO::pair(c);
        constexpr int gA = XO::gA(c), gB = XO::gB(c);
        constexpr int NK = PAIR ? 2 : 1;
        volatile T* ubc = ub + (c & 1) * (NQ * 2 * CELL_CPB);
        if (act) chunk_eval<T, TB, GRP, c>(qs, ubc, lc);
        block_sync_split();
        if (act) {
            T u[NK][NQ];
            Prim<T> w[NK];
            sfor<NK>([&](auto kk) {
                constexpr int k = decltype(kk)::value;
                sfor<NQ>([&](auto vv) {
                    constexpr int v = decltype(vv)::value;
                    u[k][v] = T(ubc[(v * 2 + k) * CELL_CPB + lc]);
                });
                w[k] = primitives(ph, u[k]);
            });
            sfor<3>([&](auto dd) {
                constexpr int d = decltype(dd)::value;
                T fs[NK][GNV];
                sfor<NK>([&](auto kk) {
                    constexpr int k = decltype(kk)::value;
                    constexpr int g = k == 0 ? gA : gB;
                    T S[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
                    if constexpr (GRP == 0 && NOISE) {
                        if (a.noise) {
                            // [direction][point][component][cell] (dg_noise.cuh)
                            const T* nb = static_cast<const T*>(a.noise);
                            const long long gc = cx.B->cell0 + cx.le, ncl = a.G.ncell;
#pragma unroll
                            for (int s = 0; s < 6; ++s) S[s] = nb[((long long)(d * NPG + g) * 6 + s) * ncl + gc];
                        } else {
                            random_stress<T>(ph, cx.B->seed, cx.nctr, 3 + d, (unsigned long long)cx.le, g, S);
                        }
                    }
                    T f[NQ];
                    point_flux<T, d>(ph, u[k], w[k], S, f);
                    sfor<GNV>([&](auto mm) { fs[k][decltype(mm)::value] = f[GV0 + decltype(mm)::value] * cx.di[d]; });
                });
                sfor<NB>([&](auto bb) {
                    constexpr int b = decltype(bb)::value;
                    constexpr double cA = vtab<TB, d>(gA, b), cB = vtab<TB, d>(gB, b);
                    static_assert(cB == cA || cB == -cA, "volume table not mirror-symmetric in x");
                    if constexpr (cA != 0.0) {
                        sfor<GNV>([&](auto mm) {
                            constexpr int m = decltype(mm)::value;
                            T fc;
                            if constexpr (!PAIR) fc = fs[0][m];
                            else if constexpr (cB == cA) fc = fs[0][m] + fs[NK - 1][m];
                            else fc = fs[0][m] - fs[NK - 1][m];
                            acc[m][b] = fma(T(cA), fc, acc[m][b]);
                        });
                    }
                });
            });
            // sources nonlinear in the state, by quadrature (ivis 2: sources.f90:51-69)
            if (GRP == 1 && ph.ivis == 2) {
                T s[NK][6];
                sfor<NK>([&](auto kk) { ten_moment_source<T>(ph, w[decltype(kk)::value], s[decltype(kk)::value]); });
                sfor<NB>([&](auto bb) {
                    constexpr int b = decltype(bb)::value;
                    constexpr double cA = TB::SRC(gA, b), cB = TB::SRC(gB, b);
                    static_assert(cB == cA || cB == -cA, "source table not mirror-symmetric in x");
                    if constexpr (cA != 0.0) {
                        sfor<6>([&](auto mm) {
                            constexpr int m = decltype(mm)::value;
                            T sc;
                            if constexpr (!PAIR) sc = s[0][m];
                            else if constexpr (cB == cA) sc = s[0][m] + s[NK - 1][m];
                            else sc = s[0][m] - s[NK - 1][m];
                            acc[m][b] = fma(T(cA), sc, acc[m][b]);
                        });
                    }
                });
            }
        }
    });
    if (!act) return;
    // the body force (no reference counterpart) is linear in the state: its
    // projection is the same linear map of the coefficients (src_gram is the
    // identity); the stress group's linear source (ivis 0) is in
    // cell_volume_linear_stress
    static_assert(src_gram_is_identity<TB>(), "source projection of a linear field is not the identity");
    if (GRP == 0 && ph.body_force != 0.0) {
        const T bf = PHC(T, ph, body_force);
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            acc[MX][b] = fma(bf, T(qs[(b * NQ + RH) * CELL_CPB + lc]), acc[MX][b]);
            acc[EN][b] = fma(bf, T(qs[(b * NQ + MX) * CELL_CPB + lc]), acc[EN][b]);
        });
    }
}

template <class T>
__device__ __forceinline__ void cell_store(const CellArgs& a, CellCtx<T>& cx, int grp, int v, int b, T e) {
    const bool stash = a.split_source != 0;
    if (stash) cx.qs[(b * NQ + v) * CELL_CPB + cx.lc] = e;   // the split source step reads them
    if (grp == 1 && stash) return;                          // stress: stored after the source step
    T o = e;
    if (a.comb != COMB_NONE) o = rk_combine(a.comb, cx.q0b[(long long)(b * NQ + v) * cx.nc + cx.le], o);
    if (b == 0 && o != o) cx.bad = true;
    cx.ob[(long long)(b * NQ + v) * cx.nc + cx.le] = o;
}

// the minus and plus face of local cell le in each direction and the face
// count of each direction of box B (periodic directions wrap the plus face)
__device__ __forceinline__ void cell_faces(const Box& B, long long le, long long (&fm)[3], long long (&fp)[3],
                                           long long (&nfd)[3]) {
    const int n0 = B.n[0], n1 = B.n[1];
    const unsigned leu = (unsigned)le, t = leu / (unsigned)n0;   // fewer than 2^31 cells per box
    const int c[3] = {(int)(leu - t * (unsigned)n0), (int)(t % (unsigned)n1), (int)(t / (unsigned)n1)};
    for (int d = 0; d < 3; ++d) {
        const int e0 = d == 0 ? B.nfp[0] : B.n[0], e1 = d == 1 ? B.nfp[1] : B.n[1], e2 = d == 2 ? B.nfp[2] : B.n[2];
        nfd[d] = (long long)e0 * e1 * e2;
        int hi = c[d] + 1;
        if (B.nfp[d] == B.n[d] && hi == B.n[d]) hi = 0;
        int a0 = d == 0 ? c[d] : c[0], a1 = d == 1 ? c[d] : c[1], a2 = d == 2 ? c[d] : c[2];
        fm[d] = (long long)a0 + (long long)e0 * (a1 + (long long)e1 * a2);
        a0 = d == 0 ? hi : c[0]; a1 = d == 1 ? hi : c[1]; a2 = d == 2 ? hi : c[2];
        fp[d] = (long long)a0 + (long long)e0 * (a1 + (long long)e1 * a2);
    }
}

// the surface sums of variable v of one cell (flux.f90:958-978) added to
// r[b]: the fluxes of its plus and minus face of each direction
template <class T, class TB>
__device__ __forceinline__ void surface_add(const T* __restrict__ flux, const Box& B, const long long (&fm)[3],
                                            const long long (&fp)[3], const long long (&nfd)[3], int v,
                                            T (&r)[TB::NB]) {
    constexpr int NB = TB::NB, NF = TB::NF;
    sfor<3>([&](auto dd) {
        constexpr int d = decltype(dd)::value;
        using FO = FOrbit<TB>;
        static_assert(face_tables_symmetric<TB, d, true>(), "surface tables not mirror-symmetric");
        const T* fb = flux + B.fbase[d] + (long long)v * NF * nfd[d];
        if constexpr (!std::is_same<T, double>::value) {
            // FP32 (not bound by its arithmetic): the two faces of a point
            // only, which keeps the register footprint of the FP32 kernels
            sfor<NF>([&](auto pp) {
                constexpr int p = decltype(pp)::value;
                const T Fp = __ldg(fb + (long long)p * nfd[d] + fp[d]);
                const T Fm = __ldg(fb + (long long)p * nfd[d] + fm[d]);
                const T Fs = Fp + Fm, Fd = Fp - Fm;
                sfor<NB>([&](auto bb) {
                    constexpr int b = decltype(bb)::value;
                    constexpr double cp = stab<TB, d, 1>(p, b), cm = stab<TB, d, 0>(p, b);
                    if constexpr (cp != 0.0) r[b] = fma(T(cp), cm == cp ? Fs : Fd, r[b]);
                });
            });
            return;
        }
        // the weights of the plus and minus faces at a tangential mirror pair
        // of points are +-one value (the parity of the function along d and
        // along the mirror): one product per chunk with a signed sum of the
        // four fluxes
        sfor<FO::NCH>([&](auto cc) {
            constexpr int c = decltype(cc)::value;
            constexpr int pA = FO::pA(c), pB = FO::pB(c);
            const T FpA = __ldg(fb + (long long)pA * nfd[d] + fp[d]);
            const T FmA = __ldg(fb + (long long)pA * nfd[d] + fm[d]);
            const T XsA = FpA + FmA, XdA = FpA - FmA;
            T X[4];
            if constexpr (FO::pair(c)) {
                const T FpB = __ldg(fb + (long long)pB * nfd[d] + fp[d]);
                const T FmB = __ldg(fb + (long long)pB * nfd[d] + fm[d]);
                const T XsB = FpB + FmB, XdB = FpB - FmB;
                X[0] = XsA + XsB; X[1] = XdA + XdB; X[2] = XsA - XsB; X[3] = XdA - XdB;
            } else {
                X[0] = XsA; X[1] = XdA; X[2] = T(0); X[3] = T(0);
            }
            sfor<NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                constexpr int k = face_class<TB, d, true>(c, b);
                if constexpr (k >= 0) r[b] = fma(T(stab<TB, d, 1>(pA, b)), X[k], r[b]);
            });
        });
    });
}

// phase 2: surface assembly (flux.f90:958-978), update and RK combination,
// one variable at a time
template <class T, class TB, int GRP>
__device__ __forceinline__ void cell_surface_update(const CellArgs& a, CellCtx<T>& cx, const T* __restrict__ flux,
                                                    T (&acc)[6][TB::NB]) {
    constexpr int NB = TB::NB, NF = TB::NF;
    constexpr int GV0 = GRP == 0 ? 0 : PXX;
    constexpr int GNV = GRP == 0 ? 5 : 6;
    const Phys& ph = a.ph;
    T* qs = cx.qs;
    const int lc = cx.lc;
    const T dt = cx.dt, faci = cx.faci;
    sfor_seq<GNV>([&](auto mm) {
        constexpr int m = decltype(mm)::value;
        constexpr int v = GV0 + m;
        T r[NB];
        sfor<NB>([&](auto bb) { r[decltype(bb)::value] = -acc[m][decltype(bb)::value]; });
        surface_add<T, TB>(flux, *cx.B, cx.fm, cx.fp, cx.nfd, v, r);
        // r[b] = glflux - source of variable v
        if (a.mode == MODE_RHS) {
            sfor<NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                cx.ob[(long long)(b * NQ + v) * cx.nc + cx.le] = r[b];
            });
            return;
        }
        if constexpr (GRP == 1 && m < 3) {
            if (ph.ivis == 2) {
                // keep R of pxx, pyy, pzz in the accumulator rows (no longer needed)
                sfor<NB>([&](auto bb) { acc[m][decltype(bb)::value] = r[decltype(bb)::value]; });
                if constexpr (m == 2) {
                    // integrator.f90:207-218: trace-coupled semi-implicit update
                    const T coll = PHC(T, ph, coll), c1d3 = T(1.0 / 3.0);
                    sfor<NB>([&](auto bb) {
                        constexpr int b = decltype(bb)::value;
                        const T q0 = qs[(b * NQ + PXX) * CELL_CPB + lc], q1 = qs[(b * NQ + PYY) * CELL_CPB + lc];
                        const T q2 = qs[(b * NQ + PZZ) * CELL_CPB + lc];
                        const T Q_sum = coll * dt * (q0 + q1 + q2) * c1d3;
                        const T R_sum = coll * (dt * dt) * (acc[0][b] + acc[1][b] + acc[2][b]) * c1d3;
                        const T e0 = faci * (q0 - dt * acc[0][b] + Q_sum - R_sum);
                        const T e1 = faci * (q1 - dt * acc[1][b] + Q_sum - R_sum);
                        const T e2 = faci * (q2 - dt * acc[2][b] + Q_sum - R_sum);
                        cell_store(a, cx, GRP, PXX, b, e0);
                        cell_store(a, cx, GRP, PYY, b, e1);
                        cell_store(a, cx, GRP, PZZ, b, e2);
                    });
                }
                return;
            }
        }
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            T e = qs[(b * NQ + v) * CELL_CPB + lc] - dt * r[b];     // integrator.f90:147-149,171-173
            if (GRP == 1 && (ph.ivis == 1 || ph.ivis == 2)) e = faci * e;   // :174,220-224
            cell_store(a, cx, GRP, v, b, e);
        });
    });
}

// phase 3 (Grad closure with RK2): implicit relaxation of E_ij with the
// sources of the advected state (ten_moment.f90:719-793 source_calc,
// :839-892 advance_time_level_source), then the RK combination and the store
template <class T, class TB>
__device__ __forceinline__ void cell_split_source(const CellArgs& a, CellCtx<T>& cx) {
    constexpr int NB = TB::NB, NPG = TB::NPG;
    const Phys& ph = a.ph;
    const volatile T* qs = cx.qs;
    const int lc = cx.lc;
    const T dt = cx.dt;
    T src[6][NB];
    sfor<6>([&](auto mm) { sfor<NB>([&](auto bb) { src[decltype(mm)::value][decltype(bb)::value] = T(0); }); });
    const T coll = PHC(T, ph, coll), oth = T(1.0 / 3.0);
    sfor_seq<NPG>([&](auto gg) {
        constexpr int g = decltype(gg)::value;
        T u[4];
        sfor<4>([&](auto vv) {
            constexpr int v = decltype(vv)::value;
            T s = T(0);
            sfor<NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                constexpr double c = TB::INT(g, b);
                if constexpr (c != 0.0) s = fma(T(c), qs[(b * NQ + v) * CELL_CPB + lc], s);
            });
            u[v] = s;
        });
        const T dni = T(1) / u[RH];
        const T vx = u[MX] * dni, vy = u[MY] * dni, vz = u[MZ] * dni, cd = coll * u[RH];
        T S[6];
        S[0] = cd * (T(2) * vx * vx - vy * vy - vz * vz) * oth;
        S[1] = cd * (T(2) * vy * vy - vz * vz - vx * vx) * oth;
        S[2] = cd * (T(2) * vz * vz - vx * vx - vy * vy) * oth;
        S[3] = cd * vx * vy;
        S[4] = cd * vx * vz;
        S[5] = cd * vy * vz;
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            constexpr double c = TB::SRC(g, b);
            if constexpr (c != 0.0) {
                sfor<6>([&](auto mm) {
                    constexpr int m = decltype(mm)::value;
                    src[m][b] = fma(T(c), S[m], src[m][b]);
                });
            }
        });
    });
    const T den = T(1) + dt * coll;
    sfor<NB>([&](auto bb) {
        constexpr int b = decltype(bb)::value;
        T E[6];
        sfor<6>([&](auto mm) { E[decltype(mm)::value] = qs[(b * NQ + PXX + decltype(mm)::value) * CELL_CPB + lc]; });
        const T Esum = coll * dt * (E[0] + E[1] + E[2]) * oth;
        const T Ssum = coll * (dt * dt) * (src[0][b] + src[1][b] + src[2][b]) * oth;
        sfor<6>([&](auto mm) {
            constexpr int m = decltype(mm)::value;
            const int v = PXX + m;
            T o = m < 3 ? (E[m] + dt * src[m][b] + Esum + Ssum) / den : (E[m] + dt * src[m][b]) / den;
            if (a.comb != COMB_NONE) o = rk_combine(a.comb, cx.q0b[(long long)(b * NQ + v) * cx.nc + cx.le], o);
            if (b == 0 && o != o) cx.bad = true;
            cx.ob[(long long)(b * NQ + v) * cx.nc + cx.le] = o;
        });
    });
}

// resident blocks per SM the register allocation must allow: FP32 fits 16
// warps per SM in 128 registers; FP64 trades occupancy for the accumulator
// rows of the larger bases
template <class T, int NB>
struct CellMinBlocks {
    static constexpr int value = std::is_same<T, float>::value ? (NB <= 4 ? 8 : NB <= 8 ? 6 : 5)
                                                               : (NB <= 4 ? 6 : NB <= 8 ? 5 : 4);
};

// SPLIT: the volume phase only; the volume terms go to a.accbuf and
// k_update adds the surface sums and does the update, one thread per
// (cell, variable), so the surface phase runs at full occupancy (ivis 0/1;
// the same operations in the same order, so the same bits)
template <class T, class TB, bool NOISE, bool SPLIT>
__global__ void __launch_bounds__(2 * CELL_CPB, (CellMinBlocks<T, TB::NB>::value))
    k_cell(const T* Qin, const T* Q0, T* out, const T* __restrict__ flux, CellArgs a) {
    pdl_enter();
    // Qin, Q0 and out may alias (the RK stages write in place); every element
    // is read before the thread that owns it writes it.
    constexpr int NB = TB::NB;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    const int grp = tid / CELL_CPB;                   // 0 hydro, 1 stress (warp-uniform)
    CellCtx<T> cx;
    cx.qs = reinterpret_cast<T*>(smem_raw);           // [NB*NQ][CELL_CPB]
    cx.ub = cx.qs + NB * NQ * CELL_CPB;               // [2][NQ][2][CELL_CPB]
    cx.lc = tid % CELL_CPB;
    const long long gc = (long long)blockIdx.x * CELL_CPB + cx.lc;
    cx.act = gc < a.G.ncell;
    cx.bx = 0; cx.le = 0; cx.nc = 1;
    if (cx.act) {
        cx.bx = box_of_cell(a.G, gc);
        cx.le = gc - a.G.boxes[cx.bx].cell0;
        cx.nc = a.G.boxes[cx.bx].ncell;
    }
    cx.B = &a.G.boxes[cx.bx];
    const Box& B = *cx.B;
    // ---- phase 0: each thread loads its own variables of its cell
    if (cx.act) {
        const T* Qb = Qin + B.q0;
        const int v0 = grp == 0 ? 0 : PXX, v1 = grp == 0 ? PXX : NQ;
        for (int v = v0; v < v1; ++v)
#pragma unroll
            for (int b = 0; b < NB; ++b) cx.qs[(b * NQ + v) * CELL_CPB + cx.lc] = Qb[(long long)(b * NQ + v) * cx.nc + cx.le];
    }
    for (int d = 0; d < 3; ++d) cx.di[d] = T(B.di[d]);
    cx.noise = a.ph.llns != 0;
    cx.nctr = NoiseCtr{cx.noise ? *a.step : 0ull, a.stage};
    cx.dt = cx.act ? T(a.st[cx.bx].dt) : T(0);
    cx.faci = T(1) / (T(1) + cx.dt * PHC(T, a.ph, coll));
    cx.ob = out + B.q0;
    cx.q0b = Q0 ? Q0 + B.q0 : nullptr;
    cx.bad = false;
    for (int d = 0; d < 3; ++d) { cx.fm[d] = 0; cx.fp[d] = 0; cx.nfd[d] = 1; }
    if (cx.act) cell_faces(B, cx.le, cx.fm, cx.fp, cx.nfd);
    __syncthreads();

    T acc[6][NB];
#pragma unroll
    for (int m = 0; m < 6; ++m)
#pragma unroll
        for (int b = 0; b < NB; ++b) acc[m][b] = T(0);
    // every thread runs the volume phase: it holds one block barrier per orbit
    if (grp == 0) cell_volume<T, TB, 0, NOISE>(a, cx, acc);
    else cell_volume<T, TB, 1, NOISE>(a, cx, acc);
    if constexpr (SPLIT) {
        // [variable][basis][cell of the grid]
        if (cx.act) {
            T* ab = static_cast<T*>(a.accbuf);
            const long long ncl = a.G.ncell;
            const int v0 = grp == 0 ? 0 : PXX, nv = grp == 0 ? 5 : 6;
#pragma unroll
            for (int m = 0; m < 6; ++m)
                if (m < nv) {
#pragma unroll
                    for (int b = 0; b < NB; ++b) ab[((long long)(v0 + m) * NB + b) * ncl + gc] = acc[m][b];
                }
        }
        return;
    }
    __syncthreads();   // every read of the other group's coefficients is done
    if (cx.act) {
        if (grp == 0) cell_surface_update<T, TB, 0>(a, cx, flux, acc);
        else cell_surface_update<T, TB, 1>(a, cx, flux, acc);
    }
    if (a.split_source) {
        __syncthreads();   // the hydro thread's updated rho and momenta are in the column
        if (grp == 1 && cx.act) cell_split_source<T, TB>(a, cx);
    }
    if (cx.bad) a.flags[0] |= FLAG_NONFINITE;   // integrator.f90:234-250 (the reference exits)
}

// k_update: the second half of a split k_cell (ivis 0/1).  r = surface sums
// - volume terms, then the forward-Euler update (integrator.f90:147-149,171-174),
// the RK combination and the NaN check of the cell average, as
// cell_surface_update does.
//
// Without the limiter: thread per (cell, variable), blockIdx.y = variable.
// With it (k_update_limit, FP64 stages whose output is the next stage's
// input): a block of UPD_CPB cells x NQ variables whose rh..en outputs go
// through shared memory to the next stage's positivity limiter (k_limit's
// operations, flux.f90:1077-1164), one thread per cell, before they are
// stored: the reference limits that stage's input in place (integrator.f90:110).
constexpr int UPD_TPB = 128;       // default threads per block of k_update
constexpr int UPD_TPB_MAX = 256;
constexpr int UPD_CPB = 16;

// the limiter's full evaluation on rows in shared memory, out of line: the
// bound check clears almost every cell, and inlined this rare path would set
// the register allocation of the whole update kernel
template <class TB, class T>
__device__ __noinline__ void limit_rows_smem(const Phys& ph, T* p, int row, int col) {
    StridedRows<T> q{p, row, col};
    limit_cell<TB, T>(ph, q);
}

// the update of variable v of cell gc; a stage's rh..en outputs go to hyd
// (the limiter's rows, stride hcol) instead of out when hyd is not null
template <class T, class TB>
__device__ __forceinline__ void update_cell_var(const T* Qin, const T* Q0, T* out, const T* __restrict__ flux,
                                                const CellArgs& a, long long gc, int v, T* hyd, int hcol) {
    constexpr int NB = TB::NB;
    const int bx = box_of_cell(a.G, gc);
    const Box& B = a.G.boxes[bx];
    const long long le = gc - B.cell0, nc = B.ncell, ncl = a.G.ncell;
    long long fm[3], fp[3], nfd[3];
    cell_faces(B, le, fm, fp, nfd);
    const T* ab = static_cast<const T*>(a.accbuf);
    T r[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) r[b] = -ab[((long long)v * NB + b) * ncl + gc];
    surface_add<T, TB>(flux, B, fm, fp, nfd, v, r);
    T* ob = out + B.q0;
    if (a.mode == MODE_RHS) {
#pragma unroll
        for (int b = 0; b < NB; ++b) ob[(long long)(b * NQ + v) * nc + le] = r[b];
        return;
    }
    const T dt = T(a.st[bx].dt), faci = T(1) / (T(1) + dt * PHC(T, a.ph, coll));
    const T* qb = Qin + B.q0;
    const T* q0b = Q0 ? Q0 + B.q0 : nullptr;
    const bool stress_faci = v >= PXX && a.ph.ivis == 1;
    bool bad = false;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const long long ix = (long long)(b * NQ + v) * nc + le;
        T e = qb[ix] - dt * r[b];
        if (stress_faci) e = faci * e;
        T o = e;
        if (a.comb != COMB_NONE) o = rk_combine(a.comb, q0b[ix], o);
        if (b == 0 && o != o) bad = true;
        if (hyd && v < 5) hyd[(v * NB + b) * hcol] = o;
        else ob[ix] = o;
    }
    if (bad) a.flags[0] |= FLAG_NONFINITE;
}

template <class T, class TB>
__global__ void __launch_bounds__(UPD_TPB_MAX) k_update(const T* Qin, const T* Q0, T* out, const T* __restrict__ flux,
                                                       CellArgs a) {
    pdl_enter();
    const long long gc = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gc >= a.G.ncell) return;
    update_cell_var<T, TB>(Qin, Q0, out, flux, a, gc, blockIdx.y, nullptr, 0);
}

template <class T, class TB>
__global__ void __launch_bounds__(UPD_CPB * NQ, 3) k_update_limit(const T* Qin, const T* Q0, T* out,
                                                                  const T* __restrict__ flux, CellArgs a) {
    pdl_enter();
    constexpr int NB = TB::NB;
    __shared__ T hyd[5 * NB * UPD_CPB];                 // [variable][basis][cell of the block]
    const int lc = threadIdx.x, v = threadIdx.y;
    const long long gc = (long long)blockIdx.x * UPD_CPB + lc;
    const bool act = gc < a.G.ncell;
    if (act) update_cell_var<T, TB>(Qin, Q0, out, flux, a, gc, v, hyd + lc, UPD_CPB);
    __syncthreads();
    if (v != 0 || !act) return;
    StridedRows<T> q{hyd + lc, NB * UPD_CPB, UPD_CPB};
    if (!(q[RH][0] >= PHC(T, a.ph, rh_floor) && limit_bound_clear<TB, T>(a.ph, q)))
        limit_rows_smem<TB, T>(a.ph, hyd + lc, NB * UPD_CPB, UPD_CPB);
    const int bx = box_of_cell(a.G, gc);
    const Box& B = a.G.boxes[bx];
    const long long le = gc - B.cell0, nc = B.ncell;
    T* ob = out + B.q0;
#pragma unroll
    for (int w = 0; w < 5; ++w)
#pragma unroll
        for (int b = 0; b < NB; ++b) ob[(long long)(b * NQ + w) * nc + le] = q[w][b];
}

// ===========================================================================
// k_mindt: hermes.f90:145-199 get_min_dt over the cell averages, FP64.
// ===========================================================================
struct DtArgs {
    Geom G;
    Phys ph;
    BoxState* st;
    int tpb;   // cells per block (a multiple of 32 up to DT_TPB; 0 = DT_TPB)
};

template <class T>
__global__ void __launch_bounds__(DT_TPB) k_mindt(const T* __restrict__ Q, DtArgs a) {
    pdl_enter();
    const long long gc = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = gc < a.G.ncell;
    int bx = 0;
    double vmag0 = 0.0;
    if (act) {
        bx = box_of_cell(a.G, gc);
        const Box& B = a.G.boxes[bx];
        const long long le = gc - B.cell0, nc = B.ncell;
        const T* Qb = Q + B.q0;
        const double dn = (double)Qb[RH * nc + le], dni = 1.0 / dn;
        const double vx = (double)Qb[MX * nc + le] * dni, vy = (double)Qb[MY * nc + le] * dni, vz = (double)Qb[MZ * nc + le] * dni;
        double cs;
        if (a.ph.ieos == 1) cs = sqrt(a.ph.aindex * ((double)Qb[EN * nc + le] * dni - 0.5 * (vx * vx + vy * vy + vz * vz)));
        else cs = sqrt(7.2 * a.ph.P_1 * pow(dn, 6.2) + a.ph.T_floor);
        const double v0 = fmax(fmax(fabs(vx) + cs, fabs(vy) + cs), fabs(vz) + cs);
        if (v0 > 0.0 && dn > a.ph.rh_mult * a.ph.rh_floor) vmag0 = v0;   // NaN never qualifies
        if (le == nc - 1) a.st[bx].cs_last = cs;
    }
    // warp max when the warp lies in one box, else one atomic per thread
    const unsigned full = 0xffffffffu;
    const int bx0 = __shfl_sync(full, bx, 0);
    const bool same = __all_sync(full, bx == bx0 || !act);
    if (same) {
        for (int o = 16; o > 0; o >>= 1) vmag0 = fmax(vmag0, __shfl_xor_sync(full, vmag0, o));
        if ((threadIdx.x & 31) == 0 && vmag0 > 0.0) atomicMax(&a.st[bx0].vmag_bits, (unsigned long long)__double_as_longlong(vmag0));
    } else if (act && vmag0 > 0.0) {
        atomicMax(&a.st[bx].vmag_bits, (unsigned long long)__double_as_longlong(vmag0));
    }
}

}  // namespace hermes

// dg_launch.cuh -- host-side launchers of the stage kernels for one
// (T, NB, NQD) instantiation, collected in a KernelSet so the C-ABI layer can
// pick the instantiation at context creation.  Each inst_*.cu file compiles
// one instantiation (the files build in parallel).
#pragma once

#include <cuda_runtime.h>

#include "dg_kernels.cuh"
#include "dg_tile.cuh"
#include "dg_trace.cuh"

namespace hermes {

struct KernelSet {
    int elem_size;
    int nb, nqd, nf;
    cudaError_t (*prepare)();
    void (*limit)(void* Q, const Geom& G, const Phys& ph, cudaStream_t s);
    // dir 0..2: the faces of one direction; dir -1: all three in one launch
    void (*face)(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s);
    void (*cell)(const void* Qin, const void* Q0, void* out, const void* flux, const CellArgs& a, cudaStream_t s);
    void (*mindt)(const void* Q, const DtArgs& a, cudaStream_t s);
    // the CFL reduction fused with the first stage's limiter (FP64: the
    // stages after it are limited by k_update's fused limiter)
    void (*mindt_limit_any)(void* Q, const DtArgs& a, cudaStream_t s);
    // face traces into a buffer for the face kernels (FaceArgs.traces); null
    // where the face kernels evaluate the traces themselves
    void (*trace)(const void* Q, void* tr, const Geom& G, cudaStream_t s, int v0, int nv);
    // the fused stage (dg_tile.cuh) and the CFL reduction fused with the first
    // stage's limiter; null where they do not exist (nbasis 8 and 10)
    void (*tile)(const void* Qin, const void* Q0, void* out, unsigned ntiles, const TileArgs& a, cudaStream_t s);
    void (*mindt_limit)(void* Q, const DtArgs& a, cudaStream_t s);
    cudaError_t (*prepare_tile)();
};

// launchers of the fused stage of one (T, nbasis 4) instantiation (inst_tile.cu)
template <class T, bool NOISE>
struct TileLaunch {
    using TB = hermes_tab::Tab<4, 2>;
    static constexpr int FMAX = (TILE_X + 1) * TILE_Y * TILE_Z > TILE_X * TILE_Y * (TILE_Z + 1)
                                    ? (TILE_X + 1) * TILE_Y * TILE_Z : TILE_X * TILE_Y * (TILE_Z + 1);
    static size_t smem() { return tile_smem<T, TB>(FMAX); }
    static cudaError_t prepare() {
        return cudaFuncSetAttribute(k_tile<T, TB, NOISE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem());
    }
    static void tile(const void* Qin, const void* Q0, void* out, unsigned ntiles, const TileArgs& a, cudaStream_t s) {
        if (ntiles == 0) return;
        TileArgs b = a;
        b.fmax = FMAX;
        launch_k(a.c.G.pdl, k_tile<T, TB, NOISE>, ntiles, TILE_NT, smem(), s, static_cast<const T*>(Qin),
                 static_cast<const T*>(Q0), static_cast<T*>(out), b);
    }
    static void mindt_limit(void* Q, const DtArgs& a, cudaStream_t s) {
        if (a.G.ncell <= 0) return;
        const unsigned nb = (unsigned)((a.G.ncell + DT_TPB - 1) / DT_TPB);
        launch_k(a.G.pdl, k_mindt_limit<T, TB>, nb, DT_TPB, 0, s, static_cast<T*>(Q), a);
    }
};

// launchers of one (T, NB, NQD) instantiation; the stochastic-stress
// variants (NOISE) are separate kernels so the noise-free ones do not carry
// the generator's registers
template <class T, int NB, int NQD>
struct Launch {
    using TB = hermes_tab::Tab<NB, NQD>;
    static size_t cell_smem() { return (size_t)(NB * NQ + 4 * NQ) * CELL_CPB * sizeof(T); }
    // the split update (k_cell's volume phase + k_update); with the
    // stochastic stress in FP32 and, in FP64, for nbasis 4 (the basis of the
    // fluctuating-hydro ensemble), which keeps the compile time of the other
    // FP64 stochastic-stress units down
    template <bool NOISE>
    static constexpr bool has_split() { return !NOISE || std::is_same<T, float>::value || NB == 4; }
    template <bool NOISE>
    static cudaError_t prepare_cell() {
        cudaError_t e = cudaFuncSetAttribute(k_cell<T, TB, NOISE, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)cell_smem());
        if constexpr (has_split<NOISE>()) {
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(k_cell<T, TB, NOISE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)cell_smem());
        }
        return e;
    }
    static void limit(void* Q, const Geom& G, const Phys& ph, cudaStream_t s) {
        if (G.ncell <= 0) return;
        const unsigned nb = (unsigned)((G.ncell + LIMIT_TPB - 1) / LIMIT_TPB);
        launch_k(G.pdl, k_limit<T, TB>, nb, LIMIT_TPB, 0, s, static_cast<T*>(Q), G, ph);
    }
    // the trace-buffer face kernels exist for the FP64 path of nbasis 8 and 10
    // without the stochastic stress
    static constexpr bool HAS_TRACE = std::is_same<T, double>::value && NB >= 8;
    template <bool NOISE, bool TRB>
    static void face_dirs(int dir, dim3 grid, int tpb, const T* q, T* f, const FaceArgs& a, cudaStream_t s) {
        if (dir == 0) launch_k(a.G.pdl, k_face<T, TB, 0, NOISE, TRB>, grid, tpb, 0, s, q, f, a);
        else if (dir == 1) launch_k(a.G.pdl, k_face<T, TB, 1, NOISE, TRB>, grid, tpb, 0, s, q, f, a);
        else launch_k(a.G.pdl, k_face<T, TB, 2, NOISE, TRB>, grid, tpb, 0, s, q, f, a);
    }
    template <bool NOISE>
    static void face(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s) {
        const int tpb = a.tpb > 0 ? a.tpb : FACE_TPB;
        const T* q = static_cast<const T*>(Q);
        T* f = static_cast<T*>(flux);
        if (dir < 0) {
            const long long n = a.G.nface[0] > a.G.nface[1] ? (a.G.nface[0] > a.G.nface[2] ? a.G.nface[0] : a.G.nface[2])
                                                             : (a.G.nface[1] > a.G.nface[2] ? a.G.nface[1] : a.G.nface[2]);
            if (n <= 0) return;
            const dim3 grid((unsigned)((n + tpb - 1) / tpb), TB::NF, 3);
            if constexpr (HAS_TRACE && !NOISE) {
                if (a.traces) { launch_k(a.G.pdl, k_faces<T, TB, NOISE, true>, grid, tpb, 0, s, q, f, a); return; }
            }
            FaceArgs b = a;
            b.traces = nullptr;
            launch_k(a.G.pdl, k_faces<T, TB, NOISE, false>, grid, tpb, 0, s, q, f, b);
            return;
        }
        const long long n = a.G.nface[dir];
        if (n <= 0) return;
        if (a.point_loop && !a.noise && !a.traces) {
            // one thread per face, its points in a loop (k_face_pl)
            const unsigned g = (unsigned)((n + tpb - 1) / tpb);
            if (dir == 0) launch_k(a.G.pdl, k_face_pl<T, TB, 0, NOISE>, g, tpb, 0, s, q, f, a);
            else if (dir == 1) launch_k(a.G.pdl, k_face_pl<T, TB, 1, NOISE>, g, tpb, 0, s, q, f, a);
            else launch_k(a.G.pdl, k_face_pl<T, TB, 2, NOISE>, g, tpb, 0, s, q, f, a);
            return;
        }
        dim3 grid((unsigned)((n + tpb - 1) / tpb), TB::NF);
        if constexpr (HAS_TRACE && !NOISE) {
            if (a.traces) { face_dirs<NOISE, true>(dir, grid, tpb, q, f, a, s); return; }
        }
        FaceArgs b = a;
        b.traces = nullptr;
        face_dirs<NOISE, false>(dir, grid, tpb, q, f, b, s);
    }
    // the traces of the variables v0 .. v0+nv-1 (all: 0, NQ)
    static void trace(const void* Q, void* tr, const Geom& G, cudaStream_t s, int v0, int nv) {
        if constexpr (HAS_TRACE) {
            if (G.ncell <= 0 || nv <= 0) return;
            dim3 grid((unsigned)((G.ncell + TRACE_TPB - 1) / TRACE_TPB), 3 * nv);
            launch_k(G.pdl, k_trace<T, TB>, grid, TRACE_TPB, 0, s, static_cast<const T*>(Q), static_cast<T*>(tr), G, v0, nv);
        }
    }
    template <bool NOISE>
    static void cell(const void* Qin, const void* Q0, void* out, const void* flux, const CellArgs& a, cudaStream_t s) {
        if (a.G.ncell <= 0) return;
        const unsigned nb = (unsigned)((a.G.ncell + CELL_CPB - 1) / CELL_CPB);
        const T* qi = static_cast<const T*>(Qin);
        const T* q0 = static_cast<const T*>(Q0);
        T* o = static_cast<T*>(out);
        const T* f = static_cast<const T*>(flux);
        if constexpr (has_split<NOISE>()) {
            if (a.accbuf && a.ph.ivis < 2 && !a.split_source) {
                if (a.phase != 2) launch_k(a.G.pdl, k_cell<T, TB, NOISE, true>, nb, 2 * CELL_CPB, cell_smem(), s, qi, q0, o, f, a);
                if (a.phase == 1) return;
                if constexpr (std::is_same<T, double>::value) {
                    if (a.limit_out && a.mode == MODE_STAGE) {
                        const unsigned ub = (unsigned)((a.G.ncell + UPD_CPB - 1) / UPD_CPB);
                        launch_k(a.G.pdl, k_update_limit<T, TB>, ub, dim3(UPD_CPB, NQ), 0, s, qi, q0, o, f, a);
                        return;
                    }
                }
                const int ut = a.utpb > 0 ? a.utpb : UPD_TPB;
                const dim3 grid((unsigned)((a.G.ncell + ut - 1) / ut), NQ);
                launch_k(a.G.pdl, k_update<T, TB>, grid, ut, 0, s, qi, q0, o, f, a);
                return;
            }
        }
        launch_k(a.G.pdl, k_cell<T, TB, NOISE, false>, nb, 2 * CELL_CPB, cell_smem(), s, qi, q0, o, f, a);
    }
    static void mindt_limit(void* Q, const DtArgs& a, cudaStream_t s) {
        if (a.G.ncell <= 0) return;
        const unsigned nb = (unsigned)((a.G.ncell + DT_TPB - 1) / DT_TPB);
        launch_k(a.G.pdl, k_mindt_limit<T, TB>, nb, DT_TPB, 0, s, static_cast<T*>(Q), a);
    }
    static void mindt(const void* Q, const DtArgs& a, cudaStream_t s) {
        if (a.G.ncell <= 0) return;
        const int tpb = a.tpb > 0 ? a.tpb : DT_TPB;
        const unsigned nb = (unsigned)((a.G.ncell + tpb - 1) / tpb);
        launch_k(a.G.pdl, k_mindt<T>, nb, tpb, 0, s, static_cast<const T*>(Q), a);
    }
};

// Each (type, basis) instantiation is spread over four translation units
// that compile in parallel: inst_<type>_nb<N>_{face,facen,cell,celln}.cu
// (the n variants carry the stochastic stress).  kernel_set() in
// kernel_sets.cu assembles the launchers of one configuration.
using FaceFn = void (*)(int, const void*, void*, const FaceArgs&, cudaStream_t);
using CellFn = void (*)(const void*, const void*, void*, const void*, const CellArgs&, cudaStream_t);
using LimitFn = void (*)(void*, const Geom&, const Phys&, cudaStream_t);
using DtFn = void (*)(const void*, const DtArgs&, cudaStream_t);
using TraceFn = void (*)(const void*, void*, const Geom&, cudaStream_t);
using PrepFn = cudaError_t (*)();

using TileFn = void (*)(const void*, const void*, void*, unsigned, const TileArgs&, cudaStream_t);
using DtLimitFn = void (*)(void*, const DtArgs&, cudaStream_t);

// precision 64 or 32, nb 4/8/10; false if unsupported
bool kernel_set(int precision, int nb, bool noise, KernelSet* out);

// ---- adjoint of the right-hand side (FP64, one box; dg_adjoint.cuh) ----
constexpr int ADJ_TPB = 64;

// how the point-wise Jacobians are formed (the values of AdjArgs::dual)
enum AdjMode { ADJ_REV = 0, ADJ_DUAL = 1, ADJ_GEN = 2 };

struct AdjArgs {
    Geom G;
    Phys ph;
    const BoxState* st;
    int mode;       // 0: out = nu = (dR/dQ)^T mu; 1: out = mu - dt*nu
    int dual;       // AdjMode: 0 reverse sweeps, 1 their dual-number check, 2 one dual pass per column
    double* cpart;  // per-block partials of mu . dR/dcoll (ceil(ncell / ADJ_TPB)), or null
    const unsigned long long* nstep;   // stochastic stress: the step counter and stage index of the
    unsigned nstage;                   // realisation held fixed (those of the forward stage)
};

// (Q, mu, trace-adjoint scratch of 2x the face-flux size, out, args, stream)
using AdjFn = cudaError_t (*)(const double*, const double*, double*, double*, const AdjArgs&, cudaStream_t);
bool adjoint_launcher(int nb, AdjFn* out);
// (Q, lam_out, lam_in, grid, physics, stream): the positivity limiter's VJP
using LimAdjFn = cudaError_t (*)(const double*, const double*, double*, const Geom&, const Phys&, cudaStream_t);
bool limiter_adjoint_launcher(int nb, LimAdjFn* out);

}  // namespace hermes

// hermes_api.cu -- the C ABI (include/hermes_gb300.h): contexts, stage and
// step orchestration on one CUDA stream, CUDA-graph replay of whole steps.
//
// A step is (hermeshd.f90:53-62, integrator.f90:62-122):
//   k_mindt + k_dt_finalize            dt from the cell averages of q (FP64)
//   per RK stage: k_limit (in place)   prep_advance's limiter
//                 k_face x, y, z       traces, boundary ghosts, Riemann fluxes
//                 k_cell               quadrature, sources, update, RK combination
// RK2: q1 = E(q); q = (q + E(q1))/2.  RK3: q1 = E(q); q1 = 3/4 q + 1/4 E(q1);
// q = 1/3 q + 2/3 E(q1) -- the reference's arrays, with its Q_2 never needed
// because each combination is fused into the stage that produces it.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "dg_init.cuh"
#include "dg_launch.cuh"
#include "dg_noise.cuh"
#include "dg_output.cuh"
#include "hermes_gb300.h"

using namespace hermes;

namespace {

struct GraphEntry {
    const void* q;
    const void* q1;
    int steps;
    cudaGraphExec_t exec;
};

__global__ void k_set_dt(BoxState* st, int nbox, double dt) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nbox) st[b].dt = dt;
}
__global__ void k_set_t(BoxState* st, int nbox, double t) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nbox) st[b].t = t;
}
__global__ void k_set_step(unsigned long long* step, unsigned long long s) {
    step[0] = s;
    step[1] = s;
}
// dt = cflm / ((vmag + cs_last) * dxi); t += dt; one thread per box
__global__ void k_dt_finalize(const Box* __restrict__ boxes, int nbox, BoxState* st, unsigned long long* step) {
    pdl_enter();
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b == 0) { step[0] = step[1]; step[1] = step[1] + 1; }
    if (b >= nbox) return;
    const double vmag = __longlong_as_double((long long)st[b].vmag_bits);
    const double vmax = (vmag + st[b].cs_last) * boxes[b].di[0];   // hermeshd.f90:174 uses dxi only
    const double dt = boxes[b].cflm / vmax;
    st[b].dt = dt;
    st[b].t = st[b].t + dt;
    st[b].vmag_bits = 0ull;
}

// adjoint stage prologue.  The stage is E = M y, y = q_in - dt R(q_in), with
// M the semi-implicit stress factor: faci = 1/(1 + dt coll) on the stresses
// for ivis 1 (integrator.f90:174); for ivis 2 faci on the off-diagonal
// stresses and faci (I + (coll dt / 3) J) on (pxx, pyy, pzz), J the 3x3 matrix
// of ones (integrator.f90:207-224); the identity elsewhere.  M is symmetric:
// mu = M lam_out.  Per-block partial sums of lam_out . (dM/dcoll) y, which,
// since sum_d y_d = sum_d E_d on the diagonal (1 + 3 coll dt / 3 = 1 / faci),
// is lam_out . (-dt faci E) on the stresses plus, on the diagonal ones,
// lam_out_d faci (dt / 3) sum_k E_k.
__global__ void __launch_bounds__(256) k_stage_pre(const double* __restrict__ lam_out, const double* __restrict__ e_out,
                                                   double* __restrict__ mu, double* __restrict__ part, long long n,
                                                   long long ncell, int ivis, double dt, double faci, double c3) {
    __shared__ double red[256];
    const long long e = (long long)blockIdx.x * 256 + threadIdx.x;
    double c = 0.0;
    if (e < n) {
        const int v = (int)((e / ncell) % NQ);
        const bool stress = v >= PXX && (ivis == 1 || ivis == 2);
        if (ivis == 2 && v >= PXX && v <= PZZ) {
            const long long d0 = e - (long long)(v - PXX) * ncell;   // pxx of the same coefficient and cell
            const double ls = lam_out[d0] + lam_out[d0 + ncell] + lam_out[d0 + 2 * ncell];
            mu[e] = faci * fma(c3, ls, lam_out[e]);
            if (e_out) {
                const double es = e_out[d0] + e_out[d0 + ncell] + e_out[d0 + 2 * ncell];
                c = lam_out[e] * faci * fma(-dt, e_out[e], dt * (1.0 / 3.0) * es);
            }
        } else {
            mu[e] = stress ? faci * lam_out[e] : lam_out[e];
            if (stress && e_out) c = lam_out[e] * (-dt * faci * e_out[e]);
        }
    }
    red[threadIdx.x] = c;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// fixed-order sum of the partials, so the result does not depend on scheduling
__global__ void k_sum_partials(const double* __restrict__ part, int n, double* __restrict__ out) {
    __shared__ double red[256];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) s += part[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = red[0];
}

__global__ void k_dt_finalize_only(const Box* __restrict__ boxes, int nbox, BoxState* st) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbox) return;
    const double vmag = __longlong_as_double((long long)st[b].vmag_bits);
    st[b].dt = boxes[b].cflm / ((vmag + st[b].cs_last) * boxes[b].di[0]);
    st[b].vmag_bits = 0ull;
}

}  // namespace

struct hermes_ctx {
    hermes_config cfg;
    KernelSet K;
    int device = 0;
    cudaStream_t stream = nullptr;       // private stream (graph capture needs a non-legacy stream)
    cudaStream_t user_stream = nullptr;  // the caller's stream; work is ordered against it both ways
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    // hermes_advance_host's copy in: a second stream, the hydro rows first
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copy_start = nullptr, ev_copy_hydro = nullptr, ev_copy_stress = nullptr;
    cudaEvent_t pending_stress = nullptr;   // the stress rows of the stage input still arriving
    // the split update's volume kernel on a side stream, concurrent with the
    // stage's trace and face kernels (launch option cell_concurrent)
    cudaStream_t side_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool cell_concurrent = false;
    std::vector<Box> h_boxes;
    std::vector<double> h_len;           // lx, ly, lz per box
    Box* d_boxes = nullptr;
    double* d_len = nullptr;
    // conservation sums: chunk map and partials, built on first use
    int* d_cons_map = nullptr;           // chunk -> box, then box -> first chunk
    double* d_cons = nullptr;            // 5 per chunk, then 5 per box
    int cons_nchunk = 0;
    Geom G{};
    Phys ph{};
    BoxState* d_st = nullptr;
    unsigned long long* d_step = nullptr;
    int* d_flags = nullptr;
    void* d_flux = nullptr;
    size_t flux_elems = 0;
    size_t q_elems = 0;
    void* d_q[2] = {nullptr, nullptr};
    std::vector<GraphEntry> graphs;
    std::string err;
    // per-kernel event timing
    bool profiling = false;
    struct Rec { int kind; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    static constexpr int NKIND = 9;
    double prof_ms[NKIND] = {};
    long long prof_n[NKIND] = {};
    // launch shape (hermes_set_launch); 0 = the compiled defaults
    int face_tpb = 0, dt_tpb = 0, graph_steps = 1;
    int update_tpb = UPD_TPB, update_tpb_default = UPD_TPB;   // threads per block of k_update
    // stochastic stress staged in HBM by its own kernels (dg_noise.cuh)
    bool noise_staged = false;
    NoiseFn noise_fn = nullptr;
    void* d_noise_cell = nullptr;
    void* d_noise_face = nullptr;
    // face traces evaluated once per stage (dg_trace.cuh)
    void* d_traces = nullptr;
    bool face_traces = false;
    // split cell update: volume terms of k_cell for k_update
    void* d_accbuf = nullptr;
    bool split_update = false;
    // fused stage (dg_tile.cuh): first tile of each box, tile count, and a
    // third state for the RK3 stage whose output cannot overwrite its input
    long long* d_tile0 = nullptr;
    unsigned ntiles = 0;
    void* d_qs = nullptr;
    bool tile_stage = false;
    bool tile_ok_default = false;   // the autotuner tries the fused stage here
    // box lookup tables of an ensemble (Geom.cbox, Geom.fbox)
    int* d_boxtab = nullptr;
    // pinned landing place of the first box's time record and the flags read
    // back after a step (one synchronisation, no pageable staging)
    struct HostRec { BoxState st; int flags; };
    HostRec* h_rec = nullptr;
    // face kernels: 0 one launch per direction, thread per (face, point)
    // (k_face); 1 the three directions in one launch (k_faces); 2 one launch
    // per direction, thread per face looping over its points (k_face_pl)
    int face_mode = 1;
    unsigned noise_stage = 0;   // stage index of the counters hermes_rhs / euler_stage / the VJPs draw with
    // adjoint scratch, allocated on first use
    AdjFn adj = nullptr;
    double* d_tadj = nullptr;   // trace adjoints: 2 x the face-flux size
    double* d_mu = nullptr;     // M lam of a stage
    double* d_part = nullptr;   // partial sums of dL/dcoll (stage factor)
    double* d_cpart = nullptr;  // partial sums of dL/dcoll (right-hand side)
    double* d_sum = nullptr;    // the two sums
    int npart = 0;
};

namespace {

int fail(hermes_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(hermes_ctx* c, const char* what, cudaError_t e) {
    return fail(c, HERMES_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define HCK(ctx, call)                                               \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return cuda_fail((ctx), #call, e_);   \
    } while (0)

bool pick_kernels(const hermes_config& c, KernelSet& K) {
    return kernel_set(c.precision, c.nbasis, c.llns != 0, &K);
}

std::string check_config(const hermes_config& c) {
    if (!((c.nbasis == 4 && c.iquad == 2) || (c.nbasis == 8 && c.iquad == 2) || (c.nbasis == 10 && c.iquad == 3)))
        return "unsupported (nbasis, iquad): supported are (4,2), (8,2), (10,3)";
    if (c.precision != 64 && c.precision != 32) return "precision must be 64 or 32";
    if (c.nx < 1 || c.ny < 1 || c.nz < 1) return "grid dimensions must be >= 1";
    if (c.ivis < 0 || c.ivis > 3) return "ivis must be 0, 1, 2 or 3 (Grad closure)";
    if (c.ihllc < 0 || c.ihllc > 2) return "ihllc must be 0 (central/LLF), 1 (HLLC) or 2 (Roe)";
    if (c.ieos != 1 && c.ieos != 2) return "ieos must be 1 or 2";
    if (c.iorder != 2 && c.iorder != 3) return "iorder must be 2 or 3";
    for (int i = 0; i < 6; ++i)
        if (c.bc[i] < 0 || c.bc[i] > 4) return "boundary codes must be 0..4";
    for (int i = 1; i < 6; ++i)
        if (c.bc[i] == HERMES_BC_INFLOW) return "the inflow boundary is defined for the x-low face only";
    if (c.bc[0] == HERMES_BC_INFLOW && !(c.inflow_rho > 0)) return "inflow density must be positive";
    if (!(c.lx > 0 && c.ly > 0 && c.lz > 0)) return "domain lengths must be positive";
    return "";
}

double default_cflm(int iquad) {  // initialize.f90:104-122
    return iquad == 2 ? 0.14 : iquad == 3 ? 0.08 : iquad == 4 ? 0.05 : 0.14;
}

Phys make_phys(const hermes_config& c) {
    Phys p{};
    p.aindex = c.aindex;
    p.aindm1 = c.aindex - 1.0;
    p.rh_floor = c.rh_floor;
    p.T_floor = c.T_floor;
    p.P_floor = c.T_floor * c.rh_floor;
    p.rh_mult = c.rh_mult;
    p.coll = c.coll;
    p.colvis = c.colvis;
    p.P_1 = c.P_1;
    p.P_base = c.P_base;
    p.eta_sd = c.eta_sd;
    p.zeta_sd = c.zeta_sd;
    p.body_force = c.body_force;
    p.inflow_u = c.inflow_u;
    p.inflow_rho = c.inflow_rho;
    p.inflow_p = c.inflow_p;
    p.inflow_ly = c.ly;
    p.ivis = c.ivis;
    p.ieos = c.ieos;
    p.ihllc = c.ihllc;
    p.llns = c.llns ? 1 : 0;
    phys_finish(p);
    return p;
}

// geometry of nbox boxes; sizes in elements
void make_boxes(const hermes_config& c, int nbox, const int32_t* dims, const double* lengths, const uint64_t* seeds,
                int nf, std::vector<Box>& boxes, std::vector<double>& len, long long& ncell, long long nface[3],
                size_t& q_elems, size_t& flux_elems) {
    boxes.resize(nbox);
    len.resize(3 * (size_t)nbox);
    ncell = 0;
    nface[0] = nface[1] = nface[2] = 0;
    for (int i = 0; i < nbox; ++i) {
        Box& b = boxes[i];
        std::memset(&b, 0, sizeof(Box));
        b.n[0] = dims ? dims[3 * i] : c.nx;
        b.n[1] = dims ? dims[3 * i + 1] : c.ny;
        b.n[2] = dims ? dims[3 * i + 2] : c.nz;
        for (int k = 0; k < 6; ++k) b.bc[k] = c.bc[k];
        for (int d = 0; d < 3; ++d)
            b.nfp[d] = (c.bc[2 * d] == HERMES_BC_PERIODIC && c.bc[2 * d + 1] == HERMES_BC_PERIODIC) ? b.n[d] : b.n[d] + 1;
        b.ncell = (long long)b.n[0] * b.n[1] * b.n[2];
        b.cell0 = ncell;
        b.q0 = ncell * (long long)c.nbasis * NQ;
        ncell += b.ncell;
        const double L[3] = {lengths ? lengths[3 * i] : c.lx, lengths ? lengths[3 * i + 1] : c.ly,
                             lengths ? lengths[3 * i + 2] : c.lz};
        for (int d = 0; d < 3; ++d) b.di[d] = (double)b.n[d] / L[d];   // initialize.f90:317-319
        for (int d = 0; d < 3; ++d) len[3 * (size_t)i + d] = L[d];
        b.cflm = c.cflm > 0 ? c.cflm : default_cflm(c.iquad);
        b.seed = seeds ? seeds[i] : c.seed + (uint64_t)i;
        for (int d = 0; d < 3; ++d) {
            long long f = 1;
            for (int e = 0; e < 3; ++e) f *= (e == d ? b.nfp[e] : b.n[e]);
            b.face0[d] = nface[d];
            nface[d] += f;
        }
    }
    q_elems = (size_t)ncell * c.nbasis * NQ;
    // flux buffer: all x faces, then all y faces, then all z faces
    long long start[3];
    start[0] = 0;
    start[1] = nface[0] * NQ * nf;
    start[2] = start[1] + nface[1] * NQ * nf;
    flux_elems = (size_t)(start[2] + nface[2] * NQ * nf);
    for (int i = 0; i < nbox; ++i)
        for (int d = 0; d < 3; ++d) boxes[i].fbase[d] = start[d] + boxes[i].face0[d] * NQ * nf;
}

void destroy_graphs(hermes_ctx* c) {
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
}

// ---- per-kernel event timing -------------------------------------------
cudaEvent_t pool_get(hermes_ctx* c) {
    if (!c->pool.empty()) { cudaEvent_t e = c->pool.back(); c->pool.pop_back(); return e; }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
struct ProfScope {
    hermes_ctx* c;
    int kind;
    cudaEvent_t a = nullptr;
    ProfScope(hermes_ctx* c_, int kind_) : c(c_), kind(kind_) {
        if (c->profiling) { a = pool_get(c); cudaEventRecord(a, c->stream); }
    }
    ~ProfScope() {
        if (!c->profiling) return;
        cudaEvent_t b = pool_get(c);
        cudaEventRecord(b, c->stream);
        c->recs.push_back(hermes_ctx::Rec{kind, a, b});
    }
};

// NVTX range over a host-side enqueue (visible to Nsight tools; a no-op otherwise)
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

// ---- enqueue helpers ---------------------------------------------------
void enq_limit(hermes_ctx* c, void* q) {
    if (c->cfg.ieos == 1 || c->cfg.ieos == 2) {   // integrator.f90:110
        ProfScope ps(c, 1);
        c->K.limit(q, c->G, c->ph, c->stream);
    }
}
void enq_faces(hermes_ctx* c, const void* q, unsigned stage) {
    FaceArgs a{c->G, c->ph, c->d_step, stage, c->face_tpb, c->noise_staged ? c->d_noise_face : nullptr,
               c->face_traces ? c->d_traces : nullptr, c->face_mode == 2 ? 1 : 0};
    if (c->pending_stress) {
        // the copy in is still delivering the stress rows: trace the hydro
        // rows (already here) first, then wait for the rest
        if (c->face_traces) {
            ProfScope ps(c, 7);
            c->K.trace(q, c->d_traces, c->G, c->stream, 0, EN + 1);
        }
        cudaStreamWaitEvent(c->stream, c->pending_stress, 0);
        c->pending_stress = nullptr;
        if (c->face_traces) {
            ProfScope ps(c, 7);
            c->K.trace(q, c->d_traces, c->G, c->stream, EN + 1, NQ - (EN + 1));
        }
    } else if (c->face_traces) {
        ProfScope ps(c, 7);
        c->K.trace(q, c->d_traces, c->G, c->stream, 0, NQ);
    }
    if (c->face_mode == 1) {
        ProfScope ps(c, 2);
        c->K.face(-1, q, c->d_flux, a, c->stream);
        return;
    }
    for (int d = 0; d < 3; ++d) {
        ProfScope ps(c, 2 + d);
        c->K.face(d, q, c->d_flux, a, c->stream);
    }
}
// phase (split update): 0 the volume kernel and the update, 1 the volume
// kernel only, 2 the update only; stream: where it is enqueued (null: the
// context's stream)
void enq_cell(hermes_ctx* c, const void* qin, const void* q0, void* out, int mode, int comb, unsigned stage,
              int limit_out = 0, int phase = 0, cudaStream_t stream = nullptr) {
    const int split = (mode == MODE_STAGE && c->cfg.ivis == 3 && c->cfg.iorder == 2) ? 1 : 0;
    CellArgs a{c->G, c->ph, c->d_st, c->d_step, c->d_flags, stage, mode, comb, split,
               c->noise_staged ? c->d_noise_cell : nullptr, c->split_update ? c->d_accbuf : nullptr, limit_out,
               c->update_tpb, phase};
    ProfScope ps(c, 5);
    c->K.cell(qin, q0, out, c->d_flux, a, stream ? stream : c->stream);
}
// the volume kernel can run beside the trace and face kernels: it reads only
// the stage input (and the staged interior noise, drawn before the fork) and
// writes only the volume-term buffer, which the update reads after the join
bool cell_forks(const hermes_ctx* c, int mode) {
    return c->cell_concurrent && c->split_update && c->side_stream && !c->profiling && c->cfg.ivis < 2 &&
           !(mode == MODE_STAGE && c->cfg.ivis == 3 && c->cfg.iorder == 2);
}
// the staged stochastic stress of a stage: interior (cell) and face draws, or
// one of them (the other's buffer null), on the given stream (null: the context's)
void enq_noise(hermes_ctx* c, unsigned stage, bool cells = true, bool faces = true, cudaStream_t stream = nullptr) {
    if (!c->noise_staged) return;
    NoiseArgs a{c->G, c->ph, c->d_step, stage};
    ProfScope ps(c, 6);
    c->noise_fn(cells ? c->d_noise_cell : nullptr, faces ? c->d_noise_face : nullptr, a, stream ? stream : c->stream);
}
// the fused stage: out = comb(q0, E(qin)), with the next stage's limiter
// applied to out when limit_out (qin must not alias out)
void enq_tile(hermes_ctx* c, const void* qin, const void* q0, void* out, int mode, int comb, unsigned stage,
              int limit_out) {
    TileArgs a{};
    a.c = CellArgs{c->G, c->ph, c->d_st, c->d_step, c->d_flags, stage, mode, comb, 0, nullptr, nullptr};
    a.tile0 = c->d_tile0;
    a.limit_out = limit_out;
    ProfScope ps(c, 8);
    c->K.tile(qin, q0, out, c->ntiles, a, c->stream);
}
// limit_in: the stage's limiter as a pass of its own (else already applied
// by the kernel that wrote qin); limit_out: the next stage's limiter applied
// to out by k_update (FP64 split update)
void enq_stage(hermes_ctx* c, void* qin, const void* q0, void* out, int comb, unsigned stage, bool limit_in = true,
               int limit_out = 0) {
    NvtxRange r("hermes stage");
    if (limit_in) enq_limit(c, qin);
    if (c->tile_stage && qin != out) {
        enq_tile(c, qin, q0, out, MODE_STAGE, comb, stage, 0);
        return;
    }
    if (cell_forks(c, MODE_STAGE)) {
        // the interior draws and the volume kernel on the side stream, the
        // face draws, traces and face kernels on the context's stream
        cudaEventRecord(c->ev_fork, c->stream);
        cudaStreamWaitEvent(c->side_stream, c->ev_fork, 0);
        if (c->pending_stress) cudaStreamWaitEvent(c->side_stream, c->pending_stress, 0);
        enq_noise(c, stage, true, false, c->side_stream);
        enq_cell(c, qin, q0, out, MODE_STAGE, comb, stage, limit_out, 1, c->side_stream);
        cudaEventRecord(c->ev_join, c->side_stream);
        enq_noise(c, stage, false, true);
        enq_faces(c, qin, stage);
        cudaStreamWaitEvent(c->stream, c->ev_join, 0);
        enq_cell(c, qin, q0, out, MODE_STAGE, comb, stage, limit_out, 2);
        return;
    }
    enq_noise(c, stage);
    enq_faces(c, qin, stage);
    enq_cell(c, qin, q0, out, MODE_STAGE, comb, stage, limit_out);
}

// the limiter fused into the CFL reduction and into k_update: FP64 with the
// split update (the separate kernels otherwise: in FP32 the block layout of
// the limiting update kernel measured ~10 % slower on the ensemble step than
// k_update plus k_limit)
bool fused_limiter(const hermes_ctx* c) {
    return c->split_update && c->K.elem_size == (int)sizeof(double) && c->cfg.ivis < 2 && c->K.mindt_limit_any &&
           (c->cfg.ieos == 1 || c->cfg.ieos == 2);
}
void enq_mindt(hermes_ctx* c, const void* q, bool advance) {
    DtArgs a{c->G, c->ph, c->d_st, c->dt_tpb};
    ProfScope ps(c, 0);
    c->K.mindt(q, a, c->stream);
    const int nb = c->G.nbox, tpb = 128;
    if (advance) launch_k(c->G.pdl, k_dt_finalize, (nb + tpb - 1) / tpb, tpb, 0, c->stream, (const Box*)c->d_boxes, nb, c->d_st, c->d_step);
    else k_dt_finalize_only<<<(nb + tpb - 1) / tpb, tpb, 0, c->stream>>>(c->d_boxes, nb, c->d_st);
}
// a step of fused stages: the CFL reduction with the first stage's limiter,
// then one kernel per stage, each applying the next stage's limiter to its
// output (the reference limits each stage's input in place, integrator.f90:110)
void enq_step_tile(hermes_ctx* c, void* q, void* q1) {
    NvtxRange r("hermes step");
    {
        DtArgs a{c->G, c->ph, c->d_st, 0};
        ProfScope ps(c, 0);
        c->K.mindt_limit(q, a, c->stream);          // hermeshd.f90:59 get_min_dt, then limiter(Q)
        const int nb = c->G.nbox, tpb = 128;
        launch_k(c->G.pdl, k_dt_finalize, (nb + tpb - 1) / tpb, tpb, 0, c->stream, (const Box*)c->d_boxes, nb, c->d_st, c->d_step);
    }
    enq_tile(c, q, nullptr, q1, MODE_STAGE, COMB_NONE, 0, 1);          // Q_1 = lim(E(Q))
    if (c->cfg.iorder == 3) {
        enq_tile(c, q1, q, c->d_qs, MODE_STAGE, COMB_34, 1, 1);        // Q_s = lim(3/4 Q + 1/4 E(Q_1))
        enq_tile(c, c->d_qs, q, q, MODE_STAGE, COMB_13, 2, 0);         // Q = 1/3 Q + 2/3 E(Q_s)
    } else {
        enq_tile(c, q1, q, q, MODE_STAGE, COMB_HALF, 1, 0);            // Q = (Q + E(Q_1))/2
    }
}

// out_last: where the last stage writes the new state (default q; a mapped
// pinned host array for hermes_advance_host, which then needs no copy back)
void enq_step(hermes_ctx* c, void* q, void* q1, void* out_last = nullptr) {
    if (c->tile_stage) {
        enq_step_tile(c, q, q1);
        return;
    }
    void* qo = out_last ? out_last : q;
    NvtxRange r("hermes step");
    const bool fl = fused_limiter(c);
    if (fl) {
        // hermeshd.f90:59 get_min_dt on the unlimited Q, then the first stage's limiter
        DtArgs a{c->G, c->ph, c->d_st, 0};
        ProfScope ps(c, 0);
        c->K.mindt_limit_any(q, a, c->stream);
        const int nb = c->G.nbox, tpb = 128;
        launch_k(c->G.pdl, k_dt_finalize, (nb + tpb - 1) / tpb, tpb, 0, c->stream, (const Box*)c->d_boxes, nb, c->d_st, c->d_step);
    } else {
        enq_mindt(c, q, true);                                   // hermeshd.f90:59
    }
    enq_stage(c, q, nullptr, q1, COMB_NONE, 0, !fl, fl);        // Q_1 = E(Q)
    if (c->cfg.iorder == 3) {
        enq_stage(c, q1, q, q1, COMB_34, 1, !fl, fl);           // Q_1 = 3/4 Q + 1/4 E(Q_1)
        enq_stage(c, q1, q, qo, COMB_13, 2, !fl, 0);            // Q = 1/3 Q + 2/3 E(Q_1)
    } else {
        enq_stage(c, q1, q, qo, COMB_HALF, 1, !fl, 0);          // Q = (Q + E(Q_1))/2
    }
}

int launch_status(hermes_ctx* c) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, "kernel launch", e);
    return HERMES_OK;
}

// order the private stream after the caller's stream, and back
int enter(hermes_ctx* c) {
    HCK(c, cudaSetDevice(c->device));
    HCK(c, cudaEventRecord(c->ev_in, c->user_stream));
    HCK(c, cudaStreamWaitEvent(c->stream, c->ev_in, 0));
    return HERMES_OK;
}
int leave(hermes_ctx* c, int rc) {
    if (cudaEventRecord(c->ev_out, c->stream) != cudaSuccess ||
        cudaStreamWaitEvent(c->user_stream, c->ev_out, 0) != cudaSuccess) {
        cudaGetLastError();
        if (rc == HERMES_OK) return fail(c, HERMES_ERR_CUDA, "stream ordering");
    }
    return rc;
}

// enqueue the copies of the first box's time record and the flags into the
// pinned record (allocated on first use)
int enq_record(hermes_ctx* c) {
    if (!c->h_rec) HCK(c, cudaMallocHost(reinterpret_cast<void**>(&c->h_rec), sizeof(hermes_ctx::HostRec)));
    HCK(c, cudaMemcpyAsync(&c->h_rec->st, c->d_st, sizeof(BoxState), cudaMemcpyDeviceToHost, c->stream));
    HCK(c, cudaMemcpyAsync(&c->h_rec->flags, c->d_flags, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    return HERMES_OK;
}

// after the stream has been synchronised: time, time step and the NaN flag
int take_record(hermes_ctx* c, double* t, double* dt) {
    if (t) *t = c->h_rec->st.t;
    if (dt) *dt = c->h_rec->st.dt;
    if (c->h_rec->flags & FLAG_NONFINITE) {
        HCK(c, cudaMemsetAsync(c->d_flags, 0, sizeof(int), c->stream));
        return fail(c, HERMES_ERR_NONFINITE, "NaN cell average produced by the step (integrator.f90:234-250)");
    }
    return HERMES_OK;
}

int read_back(hermes_ctx* c, double* t, double* dt) {
    BoxState s0;
    int flags = 0;
    int rc = enq_record(c);
    if (rc) return rc;
    HCK(c, cudaStreamSynchronize(c->stream));
    s0 = c->h_rec->st;
    flags = c->h_rec->flags;
    if (t) *t = s0.t;
    if (dt) *dt = s0.dt;
    if (flags & FLAG_NONFINITE) {
        HCK(c, cudaMemsetAsync(c->d_flags, 0, sizeof(int), c->stream));
        return fail(c, HERMES_ERR_NONFINITE, "NaN cell average produced by the step (integrator.f90:234-250)");
    }
    return HERMES_OK;
}

// a graph of `steps` whole steps on (q, q1), captured on first use
int get_graph(hermes_ctx* c, void* q, void* q1, int steps, cudaGraphExec_t* out) {
    for (auto& g : c->graphs)
        if (g.q == q && g.q1 == q1 && g.steps == steps) { *out = g.exec; return HERMES_OK; }
    cudaGraph_t graph;
    HCK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < steps; ++k) enq_step(c, q, q1);
    cudaError_t le = cudaGetLastError();
    cudaError_t ee = cudaStreamEndCapture(c->stream, &graph);
    if (le != cudaSuccess) { if (ee == cudaSuccess) cudaGraphDestroy(graph); return cuda_fail(c, "launch in capture", le); }
    HCK(c, ee);
    cudaGraphExec_t exec;
    cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    HCK(c, ie);
    if (c->graphs.size() >= 8) destroy_graphs(c);
    c->graphs.push_back(GraphEntry{q, q1, steps, exec});
    *out = exec;
    return HERMES_OK;
}

int create_impl(const hermes_config* cfg, int nbox, const int32_t* dims, const double* lengths, const uint64_t* seeds,
                void* stream, hermes_ctx** out) {
    if (!cfg || !out) return HERMES_ERR_ARG;
    *out = nullptr;
    std::string msg = check_config(*cfg);
    if (!msg.empty()) { fprintf(stderr, "hermes_create: %s\n", msg.c_str()); return HERMES_ERR_CONFIG; }
    if (nbox < 1) return HERMES_ERR_ARG;
    if ((nbox > 1 || dims) && cfg->bc[0] == HERMES_BC_INFLOW) {
        fprintf(stderr, "hermes_create: the inflow boundary takes a single grid\n");
        return HERMES_ERR_CONFIG;
    }
    if (dims)
        for (int i = 0; i < 3 * nbox; ++i)
            if (dims[i] < 1) return HERMES_ERR_CONFIG;
    // index arithmetic inside a box is 32-bit: fewer than 2^31 cells and faces per box
    for (int i = 0; i < nbox; ++i) {
        const long long n0 = dims ? dims[3 * i] : cfg->nx, n1 = dims ? dims[3 * i + 1] : cfg->ny,
                        n2 = dims ? dims[3 * i + 2] : cfg->nz;
        if ((n0 + 1) * (n1 + 1) * (n2 + 1) >= (1ll << 31)) {
            fprintf(stderr, "hermes_create: a box holds 2^31 cells or faces or more\n");
            return HERMES_ERR_SHAPE;
        }
    }
    hermes_ctx* c = new (std::nothrow) hermes_ctx();
    if (!c) return HERMES_ERR_ALLOC;
    c->cfg = *cfg;
    pick_kernels(*cfg, c->K);
    cudaGetDevice(&c->device);
    c->ph = make_phys(*cfg);
    long long ncell, nface[3];
    make_boxes(*cfg, nbox, dims, lengths, seeds, c->K.nf, c->h_boxes, c->h_len, ncell, nface, c->q_elems, c->flux_elems);
    c->G.nbox = nbox;
    // face kernels, as measured: FP64 with the three directions in one launch
    // (they fill each other's tails; TGV 64^3 nb 4: 7.52 ms against 7.57 with
    // one launch per direction and 7.73 with the point loop); FP32 nb 8/10
    // with a thread per face point (the merged kernel spills under FP32's
    // register cap); FP32 nb 4 with a thread per face looping over its points
    // (ensemble 37.4 against 37.8 ms, TGV 0.73 against 0.83 ms) where the grid
    // fills the GPU -- on a small grid that loop is latency-bound (FP64 Sod 256:
    // 0.27 s against 0.13 s with a thread per face point), so below 2^15 cells
    // a thread per face point
    c->face_mode = cfg->precision == 64 ? 1 : (cfg->nbasis == 4 && ncell >= (1ll << 15)) ? 2 : 0;
    // k_update: 64 threads per block in FP32 (measured 4 % faster on the 128^2 vortex step), 128 in FP64
    c->update_tpb_default = c->update_tpb = cfg->precision == 32 ? 64 : UPD_TPB;
    // the volume kernel beside the face kernels (measured: FP64 vortex 128^2
    // 1.446 against 1.541 ms per step, FP32 0.307 against 0.350; neutral on
    // the FP32 ensemble)
    c->cell_concurrent = true;
    c->G.pdl = 0;   // programmatic dependent launch measured neutral here: an autotuned option
    c->G.ncell = ncell;
    for (int d = 0; d < 3; ++d) c->G.nface[d] = nface[d];
    c->G.face0_dir[0] = 0;
    c->G.face0_dir[1] = nface[0];
    c->G.face0_dir[2] = nface[0] + nface[1];
    auto bail = [&](int code) { hermes_destroy(c); return code; };
    c->user_stream = static_cast<cudaStream_t>(stream);
    {
        cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming);
        if (e != cudaSuccess) { fprintf(stderr, "hermes_create: %s\n", cudaGetErrorString(e)); return bail(HERMES_ERR_CUDA); }
    }
    {
        cudaError_t e = cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
        if (e != cudaSuccess) { fprintf(stderr, "hermes_create: %s\n", cudaGetErrorString(e)); return bail(HERMES_ERR_CUDA); }
    }
    if (cudaMalloc(&c->d_boxes, sizeof(Box) * nbox) != cudaSuccess ||
        cudaMalloc(&c->d_st, sizeof(BoxState) * nbox) != cudaSuccess ||
        cudaMalloc(&c->d_step, sizeof(unsigned long long) * 2) != cudaSuccess ||
        cudaMalloc(&c->d_flags, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&c->d_flux, c->flux_elems * c->K.elem_size) != cudaSuccess) {
        cudaGetLastError();
        fprintf(stderr, "hermes_create: device allocation of %zu bytes failed\n", c->flux_elems * c->K.elem_size);
        return bail(HERMES_ERR_ALLOC);
    }
    c->G.boxes = c->d_boxes;
    if (nbox > 1) {
        // the box of each chunk of 32 cells and of 32 faces per direction
        std::vector<int> tab;
        auto build = [&](auto first, long long n) {
            const long long nch = (n + 31) / 32;
            int b = 0;
            for (long long k = 0; k < nch; ++k) {
                while (b + 1 < nbox && first(c->h_boxes[b + 1]) <= 32 * k) ++b;
                tab.push_back(b);
            }
            return nch;
        };
        const long long nc = build([](const Box& b) { return b.cell0; }, ncell);
        long long nf[3];
        nf[0] = build([](const Box& b) { return b.face0[0]; }, nface[0]);
        nf[1] = build([](const Box& b) { return b.face0[1]; }, nface[1]);
        nf[2] = build([](const Box& b) { return b.face0[2]; }, nface[2]);
        if (cudaMalloc(&c->d_boxtab, sizeof(int) * tab.size()) == cudaSuccess &&
            cudaMemcpy(c->d_boxtab, tab.data(), sizeof(int) * tab.size(), cudaMemcpyHostToDevice) == cudaSuccess) {
            c->G.cbox = c->d_boxtab;
            c->G.fbox[0] = c->G.cbox + nc;
            c->G.fbox[1] = c->G.fbox[0] + nf[0];
            c->G.fbox[2] = c->G.fbox[1] + nf[1];
        } else {
            cudaGetLastError();   // no room: the kernels search the boxes
            cudaFree(c->d_boxtab);
            c->d_boxtab = nullptr;
        }
    }
    if (cfg->llns && noise_launcher(cfg->precision, cfg->nbasis, &c->noise_fn)) {
        // staged stochastic stress: 18 NPG values per cell, 12 NF per face
        const size_t npg = (size_t)c->K.nqd * c->K.nqd * c->K.nqd, nf = (size_t)c->K.nf;
        const size_t es = c->K.elem_size;
        const size_t fcount = (size_t)(nface[0] + nface[1] + nface[2]);
        if (cudaMalloc(&c->d_noise_cell, (size_t)ncell * 18 * npg * es) == cudaSuccess &&
            cudaMalloc(&c->d_noise_face, fcount * 12 * nf * es) == cudaSuccess) {
            c->noise_staged = true;
        } else {
            cudaGetLastError();   // no room: the face and cell kernels draw the stress themselves
            cudaFree(c->d_noise_cell); cudaFree(c->d_noise_face);
            c->d_noise_cell = c->d_noise_face = nullptr;
        }
    }
    if (cfg->ivis < 2 && (!cfg->llns || c->K.elem_size == (int)sizeof(float) || cfg->nbasis == 4)) {
        // split cell update: NQ x nbasis volume terms per cell
        if (cudaMalloc(&c->d_accbuf, (size_t)ncell * NQ * c->K.nb * c->K.elem_size) == cudaSuccess) c->split_update = true;
        else { cudaGetLastError(); c->d_accbuf = nullptr; }   // no room: one kernel
    }
    if (c->K.tile && cfg->ivis < 2) {
        // fused stage: the tiles of every box, a third state, launch attributes
        std::vector<long long> t0(nbox + 1, 0);
        bool three_d = true;
        for (int i = 0; i < nbox; ++i) {
            const Box& b = c->h_boxes[i];
            const long long nt = (long long)((b.n[0] + TILE_X - 1) / TILE_X) * ((b.n[1] + TILE_Y - 1) / TILE_Y) *
                                 ((b.n[2] + TILE_Z - 1) / TILE_Z);
            t0[i + 1] = t0[i] + nt;
            three_d = three_d && b.n[2] >= TILE_Z;
        }
        if (t0[nbox] < (1ll << 31) && c->K.prepare_tile() == cudaSuccess &&
            cudaMalloc(&c->d_tile0, sizeof(long long) * (nbox + 1)) == cudaSuccess &&
            cudaMemcpy(c->d_tile0, t0.data(), sizeof(long long) * (nbox + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMalloc(&c->d_qs, c->q_elems * c->K.elem_size) == cudaSuccess) {
            c->ntiles = (unsigned)t0[nbox];
            // off by default: measured slower than the separate kernels on
            // every workload (register and shared-memory bound); the
            // autotuner tries it on grids at least one tile deep in z
            c->tile_ok_default = three_d;
        } else {
            cudaGetLastError();
            cudaFree(c->d_tile0); cudaFree(c->d_qs);
            c->d_tile0 = nullptr; c->d_qs = nullptr;
        }
    }
    if (c->K.trace) {
        // face traces: 2 sides x 3 directions x NQ x NF values per cell
        const size_t bytes = (size_t)ncell * 6 * NQ * c->K.nf * c->K.elem_size;
        if (cudaMalloc(&c->d_traces, bytes) == cudaSuccess) c->face_traces = true;
        else { cudaGetLastError(); c->d_traces = nullptr; }   // no room: the face kernels evaluate them
    }
    if (cudaMemcpy(c->d_boxes, c->h_boxes.data(), sizeof(Box) * nbox, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(c->d_st, 0, sizeof(BoxState) * nbox) != cudaSuccess ||
        cudaMemset(c->d_step, 0, sizeof(unsigned long long) * 2) != cudaSuccess ||
        cudaMemset(c->d_flags, 0, sizeof(int)) != cudaSuccess ||
        c->K.prepare() != cudaSuccess) {
        cudaGetLastError();
        return bail(HERMES_ERR_CUDA);
    }
    // initial dt of initialize.f90:343 is superseded by get_min_dt in step
    *out = c;
    return HERMES_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int hermes_abi_version(void) { return HERMES_ABI_VERSION; }

int hermes_config_size(void) { return (int)sizeof(hermes_config); }

int hermes_sizes(const hermes_config* cfg, size_t* q_elems, size_t* scratch_bytes) {
    if (!cfg) return HERMES_ERR_ARG;
    if (!check_config(*cfg).empty()) return HERMES_ERR_CONFIG;
    KernelSet K;
    pick_kernels(*cfg, K);
    std::vector<Box> boxes;
    std::vector<double> len;
    long long ncell, nface[3];
    size_t qe, fe;
    make_boxes(*cfg, 1, nullptr, nullptr, nullptr, K.nf, boxes, len, ncell, nface, qe, fe);
    if (q_elems) *q_elems = qe;
    if (scratch_bytes) *scratch_bytes = fe * K.elem_size;
    return HERMES_OK;
}

int hermes_create(const hermes_config* cfg, void* stream, hermes_ctx** out) {
    return create_impl(cfg, 1, nullptr, nullptr, nullptr, stream, out);
}

int hermes_ensemble_create(const hermes_config* cfg, int nbox, const int32_t* dims, const double* lengths,
                           const uint64_t* seeds, void* stream, hermes_ctx** out) {
    if (!dims) return HERMES_ERR_ARG;
    return create_impl(cfg, nbox, dims, lengths, seeds, stream, out);
}

int hermes_box_offsets(hermes_ctx* c, int64_t* offsets) {
    if (!c || !offsets) return HERMES_ERR_ARG;
    for (int i = 0; i < c->G.nbox; ++i) offsets[i] = c->h_boxes[i].q0;
    offsets[c->G.nbox] = (int64_t)c->q_elems;
    return HERMES_OK;
}

int hermes_destroy(hermes_ctx* c) {
    if (!c) return HERMES_ERR_ARG;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    destroy_graphs(c);
    for (auto& r : c->recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    for (auto e : c->pool) cudaEventDestroy(e);
    cudaFree(c->d_boxes);
    cudaFree(c->d_st);
    cudaFree(c->d_step);
    cudaFree(c->d_flags);
    cudaFree(c->d_flux);
    cudaFree(c->d_q[0]);
    cudaFree(c->d_q[1]);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->ev_in) cudaEventDestroy(c->ev_in);
    if (c->ev_out) cudaEventDestroy(c->ev_out);
    if (c->ev_copy_start) cudaEventDestroy(c->ev_copy_start);
    if (c->ev_copy_hydro) cudaEventDestroy(c->ev_copy_hydro);
    if (c->ev_copy_stress) cudaEventDestroy(c->ev_copy_stress);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->side_stream) cudaStreamDestroy(c->side_stream);
    cudaFree(c->d_tadj);
    cudaFree(c->d_mu);
    cudaFree(c->d_part);
    cudaFree(c->d_cpart);
    cudaFree(c->d_sum);
    cudaFree(c->d_len);
    cudaFree(c->d_cons_map);
    cudaFree(c->d_cons);
    cudaFree(c->d_noise_cell);
    cudaFree(c->d_noise_face);
    cudaFree(c->d_traces);
    cudaFree(c->d_accbuf);
    cudaFree(c->d_tile0);
    cudaFree(c->d_qs);
    cudaFree(c->d_boxtab);
    if (c->h_rec) cudaFreeHost(c->h_rec);
    delete c;
    return HERMES_OK;
}

const char* hermes_last_error(hermes_ctx* c) { return c ? c->err.c_str() : "null context"; }

void* hermes_stream(hermes_ctx* c) { return c ? (void*)c->stream : nullptr; }

int hermes_get_min_dt(hermes_ctx* c, const void* q, double* dt_out) {
    if (!c || !q || !dt_out) return fail(c, HERMES_ERR_ARG, "null argument");
    int rc = enter(c);
    if (rc) return rc;
    enq_mindt(c, q, false);
    rc = launch_status(c);
    if (rc) return leave(c, rc);
    BoxState s0;
    HCK(c, cudaMemcpyAsync(&s0, c->d_st, sizeof(BoxState), cudaMemcpyDeviceToHost, c->stream));
    HCK(c, cudaStreamSynchronize(c->stream));
    *dt_out = s0.dt;
    return leave(c, HERMES_OK);
}

int hermes_limiter(hermes_ctx* c, void* q) {
    if (!c || !q) return fail(c, HERMES_ERR_ARG, "null argument");
    int rc = enter(c);
    if (rc) return rc;
    c->K.limit(q, c->G, c->ph, c->stream);
    return leave(c, launch_status(c));
}

int hermes_rhs(hermes_ctx* c, void* q, void* rhs, int apply_limiter) {
    if (!c || !q || !rhs) return fail(c, HERMES_ERR_ARG, "null argument");
    if (q == rhs) return fail(c, HERMES_ERR_ARG, "rhs must not alias q");
    int rc = enter(c);
    if (rc) return rc;
    if (apply_limiter) enq_limit(c, q);
    if (c->tile_stage) {
        enq_tile(c, q, nullptr, rhs, MODE_RHS, COMB_NONE, c->noise_stage, 0);
        return leave(c, launch_status(c));
    }
    enq_noise(c, c->noise_stage);
    enq_faces(c, q, c->noise_stage);
    enq_cell(c, q, nullptr, rhs, MODE_RHS, COMB_NONE, c->noise_stage);
    return leave(c, launch_status(c));
}

int hermes_euler_stage(hermes_ctx* c, void* q_in, void* q_out, double dt) {
    if (!c || !q_in || !q_out) return fail(c, HERMES_ERR_ARG, "null argument");
    int rc = enter(c);
    if (rc) return rc;
    const int nb = c->G.nbox;
    k_set_dt<<<(nb + 127) / 128, 128, 0, c->stream>>>(c->d_st, nb, dt);
    enq_stage(c, q_in, nullptr, q_out, COMB_NONE, c->noise_stage);
    return leave(c, launch_status(c));
}

int hermes_set_time(hermes_ctx* c, double t) {
    if (!c) return HERMES_ERR_ARG;
    int rc = enter(c);
    if (rc) return rc;
    const int nb = c->G.nbox;
    k_set_t<<<(nb + 127) / 128, 128, 0, c->stream>>>(c->d_st, nb, t);
    return leave(c, launch_status(c));
}

int hermes_step(hermes_ctx* c, void* q, void* q1, void* q2, double* t, double* dt) {
    (void)q2;
    if (!c || !q || !q1) return fail(c, HERMES_ERR_ARG, "null argument");
    if (q == q1) return fail(c, HERMES_ERR_ARG, "q and q1 must be distinct arrays");
    int rc = enter(c);
    if (rc) return rc;
    if (t && c->G.nbox == 1) k_set_t<<<1, 32, 0, c->stream>>>(c->d_st, 1, *t);
    enq_step(c, q, q1);
    rc = launch_status(c);
    if (rc == HERMES_OK) rc = read_back(c, t, dt);
    return leave(c, rc);
}

namespace {
int enqueue_steps_impl(hermes_ctx* c, void* q, void* q1, int nsteps) {
    if (c->profiling) {
        for (int s = 0; s < nsteps; ++s) enq_step(c, q, q1);
        return launch_status(c);
    }
    const int k = c->graph_steps > 1 ? c->graph_steps : 1;
    if (nsteps >= k && k > 1) {
        cudaGraphExec_t exec;
        int rc = get_graph(c, q, q1, k, &exec);
        if (rc) return rc;
        for (int s = 0; s + k <= nsteps; s += k) HCK(c, cudaGraphLaunch(exec, c->stream));
    }
    const int rest = k > 1 ? nsteps % k : nsteps;
    if (rest > 0) {
        cudaGraphExec_t exec;
        int rc = get_graph(c, q, q1, 1, &exec);
        if (rc) return rc;
        for (int s = 0; s < rest; ++s) HCK(c, cudaGraphLaunch(exec, c->stream));
    }
    return HERMES_OK;
}

int advance_impl(hermes_ctx* c, void* q, void* q1, int nsteps, double* t, double* dt) {
    if (t && c->G.nbox == 1) k_set_t<<<1, 32, 0, c->stream>>>(c->d_st, 1, *t);
    int rc = launch_status(c);
    if (rc) return rc;
    rc = enqueue_steps_impl(c, q, q1, nsteps);
    if (rc) return rc;
    return read_back(c, t, dt);
}
}  // namespace

int hermes_advance(hermes_ctx* c, void* q, void* q1, void* q2, int nsteps, double* t, double* dt) {
    (void)q2;
    if (!c || !q || !q1 || nsteps < 0) return fail(c, HERMES_ERR_ARG, "bad argument");
    if (q == q1) return fail(c, HERMES_ERR_ARG, "q and q1 must be distinct arrays");
    int rc = enter(c);
    if (rc) return rc;
    return leave(c, advance_impl(c, q, q1, nsteps, t, dt));
}

int hermes_enqueue_steps(hermes_ctx* c, void* q, void* q1, int nsteps) {
    if (!c || !q || !q1 || nsteps < 0) return fail(c, HERMES_ERR_ARG, "bad argument");
    if (q == q1) return fail(c, HERMES_ERR_ARG, "q and q1 must be distinct arrays");
    int rc = enter(c);
    if (rc) return rc;
    return leave(c, enqueue_steps_impl(c, q, q1, nsteps));
}

int hermes_init_state(hermes_ctx* c, void* q, int32_t icid, uint64_t seed) {
    if (!c || !q) return fail(c, HERMES_ERR_ARG, "null argument");
    if (icid < 0 || icid > 7) return fail(c, HERMES_ERR_ARG, "icid must be 0..7 (initialcon.f90:41-69)");
    int rc = enter(c);
    if (rc) return rc;
    if (!c->d_len) {
        if (cudaMalloc(&c->d_len, sizeof(double) * c->h_len.size()) != cudaSuccess) {
            cudaGetLastError();
            return leave(c, fail(c, HERMES_ERR_ALLOC, "box lengths"));
        }
        HCK(c, cudaMemcpyAsync(c->d_len, c->h_len.data(), sizeof(double) * c->h_len.size(), cudaMemcpyHostToDevice,
                               c->stream));
    }
    InitArgs a{c->d_boxes, c->d_len, c->G.nbox, c->G.ncell, c->cfg.nbasis, icid,
               c->cfg.aindex, c->cfg.rh_floor, c->cfg.T_floor, c->cfg.P_base, (unsigned long long)seed};
    cudaError_t e = init_launch(c->cfg.precision, q, a, c->stream);
    if (e != cudaSuccess) return leave(c, cuda_fail(c, "initial-state launch", e));
    return leave(c, HERMES_OK);
}

int hermes_conserved(hermes_ctx* c, const void* q, double* sums) {
    if (!c || !q || !sums) return fail(c, HERMES_ERR_ARG, "null argument");
    int rc = enter(c);
    if (rc) return rc;
    const int nbox = c->G.nbox;
    if (!c->d_cons) {
        std::vector<int> map;
        std::vector<int> first(nbox + 1, 0);
        for (int b = 0; b < nbox; ++b) {
            first[b] = (int)map.size();
            const long long n = c->h_boxes[b].ncell;
            for (long long k = 0; k < (n + CONS_CHUNK - 1) / CONS_CHUNK; ++k) map.push_back(b);
        }
        first[nbox] = (int)map.size();
        c->cons_nchunk = (int)map.size();
        map.insert(map.end(), first.begin(), first.end());
        if (cudaMalloc(&c->d_cons_map, sizeof(int) * map.size()) != cudaSuccess ||
            cudaMalloc(&c->d_cons, sizeof(double) * 5 * ((size_t)c->cons_nchunk + nbox)) != cudaSuccess) {
            cudaGetLastError();
            return leave(c, fail(c, HERMES_ERR_ALLOC, "conservation-sum scratch"));
        }
        HCK(c, cudaMemcpy(c->d_cons_map, map.data(), sizeof(int) * map.size(), cudaMemcpyHostToDevice));
    }
    ConsArgs a{c->d_boxes, c->d_cons_map, c->d_cons_map + c->cons_nchunk, c->d_cons,
               c->d_cons + 5 * (size_t)c->cons_nchunk, c->cons_nchunk};
    cudaError_t e = cons_launch(c->cfg.precision, q, a, nbox, c->stream);
    if (e != cudaSuccess) return leave(c, cuda_fail(c, "conservation-sum launch", e));
    HCK(c, cudaMemcpyAsync(sums, a.out, sizeof(double) * 5 * nbox, cudaMemcpyDeviceToHost, c->stream));
    HCK(c, cudaStreamSynchronize(c->stream));
    return leave(c, HERMES_OK);
}

int hermes_derived(hermes_ctx* c, const void* q, float* out, int32_t nvtk, uint32_t mask,
                   const hermes_output_units* u) {
    if (!c || !q || !out || !u) return fail(c, HERMES_ERR_ARG, "null argument");
    if (nvtk < 1 || nvtk > 4) return fail(c, HERMES_ERR_ARG, "nvtk must be 1..4 (basis_funcs.f90:100-116)");
    if (mask == 0 || mask >= (1u << DV_N)) return fail(c, HERMES_ERR_ARG, "mask selects none or unknown variables");
    if (c->G.nbox != 1) return fail(c, HERMES_ERR_CONFIG, "derived fields are written per grid: use one box");
    DerivedFn fn;
    if (!derived_launcher(c->cfg.precision, c->cfg.nbasis, &fn)) return fail(c, HERMES_ERR_CONFIG, "no derived-field kernel");
    DerivedArgs a{};
    a.G = c->G;
    a.aindex = c->cfg.aindex;
    a.n0 = u->n0; a.v0 = u->v0; a.t0 = u->t0; a.te0 = u->te0; a.eV_per_K = u->eV_per_K;
    a.nvtk = nvtk;
    a.mask = mask;
    for (int v = 0, n = 0; v < DV_N; ++v) a.slot[v] = ((mask >> v) & 1u) ? n++ : 0;
    int rc = enter(c);
    if (rc) return rc;
    cudaError_t e = fn(q, out, a, c->stream);
    if (e != cudaSuccess) return leave(c, cuda_fail(c, "derived-field launch", e));
    return leave(c, HERMES_OK);
}

int hermes_set_launch(hermes_ctx* c, const hermes_launch* l) {
    if (!c || !l) return fail(c, HERMES_ERR_ARG, "null argument");
    const int f = l->face_tpb, d = l->dt_tpb, g = l->steps_per_graph;
    if (f != 0 && f != 32 && f != 64 && f != 128) return fail(c, HERMES_ERR_ARG, "face_tpb must be 0, 32, 64 or 128");
    if (d != 0 && (d < 32 || d > DT_TPB || d % 32)) return fail(c, HERMES_ERR_ARG, "dt_tpb must be 0 or a multiple of 32 up to 256");
    if (g < 0 || g > 64) return fail(c, HERMES_ERR_ARG, "steps_per_graph must be in 0..64");
    const bool staged = l->noise_inline == 0 && c->d_noise_cell != nullptr;
    if (l->noise_inline == 0 && c->cfg.llns && !c->d_noise_cell)
        return fail(c, HERMES_ERR_ALLOC, "no staged-noise buffers (device memory was short at creation)");
    if (l->face_traces != 0 && l->face_traces != 1) return fail(c, HERMES_ERR_ARG, "face_traces must be 0 or 1");
    if (l->face_traces == 1 && !c->d_traces)
        return fail(c, HERMES_ERR_ARG, "face traces need FP64, nbasis 8 or 10, no stochastic stress and room for the buffer");
    const bool traces = l->face_traces == 1;
    if (l->split_update != 0 && l->split_update != 1) return fail(c, HERMES_ERR_ARG, "split_update must be 0 or 1");
    if (l->split_update == 1 && !c->d_accbuf)
        return fail(c, HERMES_ERR_ARG, "the split update needs ivis 0/1, room for the buffer and, with the stochastic "
                                       "stress in FP64, nbasis 4");
    const bool split = l->split_update == 1;
    if (l->tile_stage != 0 && l->tile_stage != 1) return fail(c, HERMES_ERR_ARG, "tile_stage must be 0 or 1");
    if (l->tile_stage == 1 && !c->d_tile0)
        return fail(c, HERMES_ERR_ARG, "the fused stage needs nbasis 4, ivis 0/1 and room for a third state");
    const bool tile = l->tile_stage == 1;
    if (l->pdl != 0 && l->pdl != 1) return fail(c, HERMES_ERR_ARG, "pdl must be 0 or 1");
    if (l->faces_merged < 0 || l->faces_merged > 2) return fail(c, HERMES_ERR_ARG, "faces_merged must be 0, 1 or 2");
    if (l->cell_concurrent != 0 && l->cell_concurrent != 1) return fail(c, HERMES_ERR_ARG, "cell_concurrent must be 0 or 1");
    const int u = l->update_tpb ? l->update_tpb : c->update_tpb_default;
    if (u != 0 && u != 64 && u != 128 && u != 256) return fail(c, HERMES_ERR_ARG, "update_tpb must be 0, 64, 128 or 256");
    if (f != c->face_tpb || d != c->dt_tpb || staged != c->noise_staged || traces != c->face_traces ||
        split != c->split_update || tile != c->tile_stage || l->pdl != c->G.pdl ||
        l->faces_merged != c->face_mode || u != c->update_tpb || (l->cell_concurrent == 1) != c->cell_concurrent) {
        // captured graphs hold the old launch shape
        HCK(c, cudaSetDevice(c->device));
        HCK(c, cudaStreamSynchronize(c->stream));
        destroy_graphs(c);
    }
    c->face_tpb = f;
    c->dt_tpb = d;
    c->graph_steps = g > 0 ? g : 1;
    c->noise_staged = staged;
    c->face_traces = traces;
    c->split_update = split;
    c->tile_stage = tile;
    c->G.pdl = l->pdl;
    c->face_mode = l->faces_merged;
    c->update_tpb = u;
    c->cell_concurrent = l->cell_concurrent == 1;
    return HERMES_OK;
}

int hermes_get_launch(hermes_ctx* c, hermes_launch* l) {
    if (!c || !l) return fail(c, HERMES_ERR_ARG, "null argument");
    l->face_tpb = c->face_tpb > 0 ? c->face_tpb : FACE_TPB;
    l->dt_tpb = c->dt_tpb > 0 ? c->dt_tpb : DT_TPB;
    l->steps_per_graph = c->graph_steps;
    l->noise_inline = (c->cfg.llns && !c->noise_staged) ? 1 : 0;
    l->face_traces = c->face_traces ? 1 : 0;
    l->split_update = c->split_update ? 1 : 0;
    l->tile_stage = c->tile_stage ? 1 : 0;
    l->pdl = c->G.pdl;
    l->faces_merged = c->face_mode;
    l->update_tpb = c->update_tpb;
    l->cell_concurrent = c->cell_concurrent ? 1 : 0;
    return HERMES_OK;
}

int hermes_profile_enable(hermes_ctx* c, int enable) {
    if (!c) return HERMES_ERR_ARG;
    c->profiling = enable != 0;
    return HERMES_OK;
}

int hermes_profile_read(hermes_ctx* c, double* ms, int64_t* launches) {
    if (!c) return HERMES_ERR_ARG;
    HCK(c, cudaSetDevice(c->device));
    HCK(c, cudaStreamSynchronize(c->stream));
    for (auto& r : c->recs) {
        float m = 0.f;
        if (cudaEventElapsedTime(&m, r.a, r.b) == cudaSuccess) {
            c->prof_ms[r.kind] += m;
            c->prof_n[r.kind] += 1;
        }
        c->pool.push_back(r.a);
        c->pool.push_back(r.b);
    }
    c->recs.clear();
    cudaGetLastError();
    for (int k = 0; k < hermes_ctx::NKIND; ++k) {
        if (ms) ms[k] = c->prof_ms[k];
        if (launches) launches[k] = c->prof_n[k];
        c->prof_ms[k] = 0;
        c->prof_n[k] = 0;
    }
    return HERMES_OK;
}

int hermes_advance_host(hermes_ctx* c, void* q_host, int nsteps, double* t, double* dt) {
    if (!c || !q_host || nsteps < 0) return fail(c, HERMES_ERR_ARG, "bad argument");
    int rc = enter(c);
    if (rc) return rc;
    const size_t bytes = c->q_elems * c->K.elem_size;
    for (int i = 0; i < 2; ++i)
        if (!c->d_q[i] && cudaMalloc(&c->d_q[i], bytes) != cudaSuccess) {
            cudaGetLastError();
            return leave(c, fail(c, HERMES_ERR_ALLOC, "device buffers for host-array stepping"));
        }
    // pinned host memory mapped into the device's address space: the last
    // stage of the last step stores the new state into it directly, so the
    // copy back overlaps that kernel's arithmetic instead of following it
    void* q_mapped = nullptr;
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, q_host) == cudaSuccess) {
        if (pa.type == cudaMemoryTypeHost && pa.devicePointer) q_mapped = pa.devicePointer;
    } else {
        cudaGetLastError();
    }
    const bool direct = q_mapped && nsteps >= 1 && !c->tile_stage;
    // one grid in pinned memory: the copy in goes on a second stream, the
    // hydro rows (rh..en of every coefficient) first; the first step's CFL
    // reduction, limiter and hydro traces read only those and start while
    // the stress rows are still arriving (the face kernels wait for them)
    const bool split = direct && c->G.nbox == 1;
    if (split && !c->copy_stream) {
        cudaError_t e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_copy_start, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_copy_hydro, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_copy_stress, cudaEventDisableTiming);
        if (e != cudaSuccess) return leave(c, cuda_fail(c, "copy stream", e));
    }
    // copy in, step, copy the state and the time record out, one synchronisation
    if (split) {
        const size_t es = (size_t)c->K.elem_size, nc = (size_t)c->G.ncell, pitch = (size_t)NQ * nc * es;
        const size_t hydro = (size_t)(EN + 1) * nc * es;
        char* dq = static_cast<char*>(c->d_q[0]);
        const char* hq = static_cast<const char*>(q_host);
        HCK(c, cudaEventRecord(c->ev_copy_start, c->stream));
        HCK(c, cudaStreamWaitEvent(c->copy_stream, c->ev_copy_start, 0));
        HCK(c, cudaMemcpy2DAsync(dq, pitch, hq, pitch, hydro, (size_t)c->cfg.nbasis, cudaMemcpyHostToDevice,
                                 c->copy_stream));
        HCK(c, cudaEventRecord(c->ev_copy_hydro, c->copy_stream));
        HCK(c, cudaMemcpy2DAsync(dq + hydro, pitch, hq + hydro, pitch, pitch - hydro, (size_t)c->cfg.nbasis,
                                 cudaMemcpyHostToDevice, c->copy_stream));
        HCK(c, cudaEventRecord(c->ev_copy_stress, c->copy_stream));
        HCK(c, cudaStreamWaitEvent(c->stream, c->ev_copy_hydro, 0));
        c->pending_stress = c->ev_copy_stress;
    } else {
        HCK(c, cudaMemcpyAsync(c->d_q[0], q_host, bytes, cudaMemcpyHostToDevice, c->stream));
    }
    if (t && c->G.nbox == 1) k_set_t<<<1, 32, 0, c->stream>>>(c->d_st, 1, *t);
    rc = launch_status(c);
    if (rc == HERMES_OK && direct) {
        // the first step eagerly (it consumes the pending stress rows), the
        // middle ones from the graphs, the last into the host array
        if (nsteps > 1) {
            enq_step(c, c->d_q[0], c->d_q[1]);
            if (c->pending_stress) {
                cudaStreamWaitEvent(c->stream, c->pending_stress, 0);
                c->pending_stress = nullptr;
            }
            rc = launch_status(c);
            if (rc == HERMES_OK && nsteps > 2) rc = enqueue_steps_impl(c, c->d_q[0], c->d_q[1], nsteps - 2);
        }
        if (rc == HERMES_OK) {
            enq_step(c, c->d_q[0], c->d_q[1], q_mapped);
            rc = launch_status(c);
        }
    } else if (rc == HERMES_OK) {
        rc = enqueue_steps_impl(c, c->d_q[0], c->d_q[1], nsteps);
    }
    if (c->pending_stress) {   // (not consumed: wait here)
        cudaStreamWaitEvent(c->stream, c->pending_stress, 0);
        c->pending_stress = nullptr;
    }
    if (rc) return leave(c, rc);
    if (!direct) HCK(c, cudaMemcpyAsync(q_host, c->d_q[0], bytes, cudaMemcpyDeviceToHost, c->stream));
    rc = enq_record(c);
    if (rc) return leave(c, rc);
    HCK(c, cudaStreamSynchronize(c->stream));
    return leave(c, take_record(c, t, dt));
}

int hermes_box_times(hermes_ctx* c, double* t, double* dt) {
    if (!c) return HERMES_ERR_ARG;
    int rc = enter(c);
    if (rc) return rc;
    std::vector<BoxState> s(c->G.nbox);
    HCK(c, cudaMemcpyAsync(s.data(), c->d_st, sizeof(BoxState) * s.size(), cudaMemcpyDeviceToHost, c->stream));
    HCK(c, cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < s.size(); ++i) {
        if (t) t[i] = s[i].t;
        if (dt) dt[i] = s[i].dt;
    }
    return leave(c, HERMES_OK);
}

int hermes_set_noise_step(hermes_ctx* c, uint64_t step) {
    if (!c) return HERMES_ERR_ARG;
    int rc = enter(c);
    if (rc) return rc;
    k_set_step<<<1, 1, 0, c->stream>>>(c->d_step, (unsigned long long)step);
    return leave(c, launch_status(c));
}

int hermes_set_noise_stage(hermes_ctx* c, int32_t stage) {
    if (!c) return HERMES_ERR_ARG;
    if (stage < 0 || stage > 2) return fail(c, HERMES_ERR_ARG, "stage must be 0, 1 or 2");
    c->noise_stage = (unsigned)stage;
    return HERMES_OK;
}

int hermes_check(hermes_ctx* c) {
    if (!c) return HERMES_ERR_ARG;
    int rc = enter(c);
    if (rc) return rc;
    rc = launch_status(c);
    if (rc == HERMES_OK) rc = read_back(c, nullptr, nullptr);
    return leave(c, rc);
}

// ---- adjoint -------------------------------------------------------------
namespace {
std::string adjoint_unsupported(const hermes_config& c, int nbox) {
    if (c.precision != 64) return "the adjoint is FP64 only";
    if (nbox != 1) return "the adjoint takes a single grid";
    if (c.ivis < 0 || c.ivis > 2) return "the adjoint supports ivis 0, 1 and 2";
    if (c.ieos == 2 && c.ihllc == 1)
        return "the adjoint does not take HLLC with ieos 2 (its sound speed uses 1/rho of another face point)";
    if (c.bc[0] == HERMES_BC_INFLOW) return "the adjoint does not model the inflow boundary";
    for (int d = 0; d < 3; ++d)
        if ((c.bc[2 * d] == HERMES_BC_PERIODIC) != (c.bc[2 * d + 1] == HERMES_BC_PERIODIC))
            return "the adjoint needs both or neither end of a direction periodic";
    return "";
}

// the point-wise Jacobians (AdjMode): the hand-derived reverse sweeps cover
// ivis 0/1 with ieos 1 and no stochastic stress; ivis 2, the Tait equation of
// state and the stochastic stress take one dual pass per column.
// HERMES_ADJOINT_DUAL=1 selects the dual-number check of the reverse sweeps
// (those cases), =2 the per-column passes for any case.
int adjoint_mode(const hermes_config& c) {
    const char* e = std::getenv("HERMES_ADJOINT_DUAL");
    if (c.ivis == 2 || c.ieos == 2 || c.llns || (e && e[0] == '2')) return ADJ_GEN;
    return (e && e[0] == '1') ? ADJ_DUAL : ADJ_REV;
}

int adj_prepare(hermes_ctx* c) {
    const std::string why = adjoint_unsupported(c->cfg, c->G.nbox);
    if (!why.empty()) return fail(c, HERMES_ERR_CONFIG, why);
    if (!c->adj && !adjoint_launcher(c->cfg.nbasis, &c->adj)) return fail(c, HERMES_ERR_CONFIG, "no adjoint for this basis");
    if (!c->d_tadj) {
        c->npart = (int)((c->q_elems + 255) / 256);
        if (cudaMalloc(&c->d_tadj, 2 * c->flux_elems * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&c->d_mu, c->q_elems * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&c->d_part, (size_t)c->npart * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&c->d_cpart, (size_t)((c->G.ncell + ADJ_TPB - 1) / ADJ_TPB) * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&c->d_sum, 2 * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            return fail(c, HERMES_ERR_ALLOC, "adjoint scratch");
        }
    }
    return HERMES_OK;
}
}  // namespace

int hermes_rhs_vjp(hermes_ctx* c, const void* q, const void* mu, void* nu) {
    if (!c || !q || !mu || !nu) return fail(c, HERMES_ERR_ARG, "null argument");
    if (nu == q || nu == mu) return fail(c, HERMES_ERR_ARG, "nu must not alias q or mu");
    int rc = enter(c);
    if (rc) return rc;
    rc = adj_prepare(c);
    if (rc) return leave(c, rc);
    AdjArgs a{c->G, c->ph, c->d_st, 0, adjoint_mode(c->cfg), nullptr, c->d_step, c->noise_stage};
    cudaError_t e = c->adj(static_cast<const double*>(q), static_cast<const double*>(mu), c->d_tadj,
                           static_cast<double*>(nu), a, c->stream);
    if (e != cudaSuccess) return leave(c, cuda_fail(c, "adjoint launch", e));
    return leave(c, HERMES_OK);
}

int hermes_limiter_vjp(hermes_ctx* c, const void* q, const void* lam_out, void* lam_in) {
    if (!c || !q || !lam_out || !lam_in) return fail(c, HERMES_ERR_ARG, "null argument");
    if (lam_in == q) return fail(c, HERMES_ERR_ARG, "lam_in must not alias q");
    int rc = enter(c);
    if (rc) return rc;
    rc = adj_prepare(c);
    if (rc) return leave(c, rc);
    LimAdjFn fn = nullptr;
    if (!limiter_adjoint_launcher(c->cfg.nbasis, &fn)) return leave(c, fail(c, HERMES_ERR_CONFIG, "no limiter adjoint for this basis"));
    cudaError_t e = fn(static_cast<const double*>(q), static_cast<const double*>(lam_out), static_cast<double*>(lam_in),
                       c->G, c->ph, c->stream);
    if (e != cudaSuccess) return leave(c, cuda_fail(c, "limiter adjoint launch", e));
    return leave(c, HERMES_OK);
}

int hermes_stage_vjp(hermes_ctx* c, const void* q_in, const void* e_out, const void* lam_out, void* lam_in, double dt,
                     double* dcoll) {
    if (!c || !q_in || !lam_out || !lam_in) return fail(c, HERMES_ERR_ARG, "null argument");
    if (lam_in == q_in || (e_out && lam_in == e_out)) return fail(c, HERMES_ERR_ARG, "lam_in must not alias q_in or e_out");
    if (dcoll && !e_out) return fail(c, HERMES_ERR_ARG, "dcoll needs e_out");
    if (!(dt > 0.0)) return fail(c, HERMES_ERR_ARG, "dt must be positive");
    int rc = enter(c);
    if (rc) return rc;
    rc = adj_prepare(c);
    if (rc) return leave(c, rc);
    k_set_dt<<<1, 32, 0, c->stream>>>(c->d_st, 1, dt);
    const long long n = (long long)c->q_elems;
    const double faci = 1.0 / (1.0 + dt * c->cfg.coll);
    k_stage_pre<<<c->npart, 256, 0, c->stream>>>(static_cast<const double*>(lam_out), static_cast<const double*>(e_out),
                                                 c->d_mu, c->d_part, n, c->G.ncell, c->cfg.ivis, dt, faci,
                                                 c->cfg.coll * dt * (1.0 / 3.0));
    if (dcoll) k_sum_partials<<<1, 256, 0, c->stream>>>(c->d_part, c->npart, c->d_sum);
    // R depends on coll for ivis 0 and 2: the cell pass adds mu . dR/dcoll
    const bool r_coll = dcoll && (c->cfg.ivis == 0 || c->cfg.ivis == 2);
    AdjArgs a{c->G, c->ph, c->d_st, 1, adjoint_mode(c->cfg), r_coll ? c->d_cpart : nullptr, c->d_step, c->noise_stage};
    cudaError_t e = c->adj(static_cast<const double*>(q_in), c->d_mu, c->d_tadj, static_cast<double*>(lam_in), a, c->stream);
    if (e != cudaSuccess) return leave(c, cuda_fail(c, "adjoint launch", e));
    if (dcoll) {
        if (r_coll)
            k_sum_partials<<<1, 256, 0, c->stream>>>(c->d_cpart, (int)((c->G.ncell + ADJ_TPB - 1) / ADJ_TPB), c->d_sum + 1);
        double h[2] = {0.0, 0.0};
        HCK(c, cudaMemcpyAsync(h, c->d_sum, (r_coll ? 2 : 1) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        HCK(c, cudaStreamSynchronize(c->stream));
        // lam_out . dE/dcoll = lam_out . (dM/dcoll) y + (M lam_out) . (-dt dR/dcoll)
        *dcoll = h[0] - dt * h[1];
    }
    return leave(c, launch_status(c));
}

}  // extern "C"

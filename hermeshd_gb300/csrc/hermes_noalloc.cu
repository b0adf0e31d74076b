// hermes_noalloc.cu -- hermes_rhs_noalloc: the DG right-hand side of one grid
// computed without a context and without allocating device memory.
//
// Who needs it: a caller that cannot allocate device memory at the point it
// needs a right-hand side -- for example a host code whose device memory is
// reserved up front by its own framework or pool (a Fortran/MPI driver calling
// through its FFI under a fixed memory budget), or a time loop that must not
// pay cudaMalloc's device-wide synchronisation.  hermes_create allocates the
// face-flux scratch with cudaMalloc; this entry point uses a file-scope device
// array instead.
//
// The scratch is g_scratch below: HERMES_NOALLOC_SCRATCH_BYTES (64 MiB) of
// device memory that every GPU which loads this library holds until the
// process exits.  The face fluxes of the call (3 directions x faces x nQ x
// face points x element size) must fit in it; larger grids are rejected with
// HERMES_ERR_SHAPE.  All calls share the array, so calls that overlap on the
// GPU (two streams at once, or two host threads) race; serialise them on one
// stream.  Every face flux the cell kernel reads is written by the face
// kernels of the same call, so nothing of the previous call is read; the
// small records (grid descriptor, time-step record, error flag, noise
// counter) are rewritten on every call by k_noalloc_records, a one-thread
// kernel that receives the grid descriptor as a kernel parameter (by value),
// so no host memory has to outlive the call.
//
// The right-hand side is returned as computed: the reference's NaN check
// belongs to the update (integrator.f90:234-250), not to the right-hand side,
// so a non-finite value is not flagged (check the output if needed).  With the
// stochastic stress on, every call draws the realisation of step 0, stage 0
// (the Philox counters a fresh context's hermes_rhs uses).
//
// Device addresses: in host code g_scratch names a host-side stand-in, not a
// device address.  The first call on a device, with that device current,
// resolves the addresses with cudaGetSymbolAddress (checked) and caches them
// for that device; the later calls reuse them.  That first call should come
// before any stream capture.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "dg_launch.cuh"
#include "hermes_gb300.h"

using namespace hermes;

namespace {

static __device__ __align__(256) unsigned char g_scratch[HERMES_NOALLOC_SCRATCH_BYTES];
static __device__ __align__(256) Box g_box;
static __device__ __align__(16) BoxState g_state;
static __device__ __align__(16) unsigned long long g_step[2];
static __device__ __align__(16) int g_flags;

// the per-call records: the grid descriptor (a kernel parameter, so nothing
// of the host's stack is read after the call returns), a zeroed time-step
// record and error flag, and the noise counter of step 0
__global__ void k_noalloc_records(Box b) {
    g_box = b;
    g_state = BoxState{0.0, 0.0, 0ull, 0.0};
    g_step[0] = 0ull;
    g_step[1] = 0ull;
    g_flags = 0;
}

struct DevAddrs {
    bool ready = false;
    void* scratch = nullptr;
    Box* box = nullptr;
    BoxState* state = nullptr;
    unsigned long long* step = nullptr;
    int* flags = nullptr;
};

constexpr int kMaxDevices = 64;
DevAddrs g_addrs[kMaxDevices];
std::mutex g_mutex;

void set_err(char* err, size_t errlen, const char* msg) {
    if (err && errlen) {
        std::strncpy(err, msg, errlen - 1);
        err[errlen - 1] = '\0';
    }
}

// once per device, with that device current
int device_addrs(int dev, DevAddrs** out, char* err, size_t errlen) {
    if (dev < 0 || dev >= kMaxDevices) {
        set_err(err, errlen, "device ordinal out of range");
        return HERMES_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_mutex);
    DevAddrs& a = g_addrs[dev];
    if (!a.ready) {
        cudaError_t e = cudaGetSymbolAddress(&a.scratch, g_scratch);
        if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&a.box, g_box);
        if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&a.state, g_state);
        if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&a.step, g_step);
        if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&a.flags, g_flags);
        if (e != cudaSuccess) {
            set_err(err, errlen, cudaGetErrorString(e));
            return HERMES_ERR_CUDA;
        }
        a.ready = true;
    }
    *out = &a;
    return HERMES_OK;
}

bool supported(const hermes_config& c) {
    const bool basis = (c.nbasis == 4 && c.iquad == 2) || (c.nbasis == 8 && c.iquad == 2) || (c.nbasis == 10 && c.iquad == 3);
    bool ok = basis && (c.precision == 64 || c.precision == 32) && c.nx >= 1 && c.ny >= 1 && c.nz >= 1 &&
              c.ivis >= 0 && c.ivis <= 3 && c.ihllc >= 0 && c.ihllc <= 2 && (c.ieos == 1 || c.ieos == 2) && c.lx > 0 && c.ly > 0 && c.lz > 0;
    for (int i = 0; i < 6; ++i) ok = ok && c.bc[i] >= 0 && c.bc[i] <= 3;
    return ok;
}

KernelSet kernels_for(const hermes_config& c) {
    KernelSet k{};
    kernel_set(c.precision, c.nbasis, c.llns != 0, &k);
    return k;
}

}  // namespace

extern "C" int hermes_rhs_noalloc(const hermes_config* cfg, void* q, void* rhs, int apply_limiter, void* stream,
                                  char* err, size_t errlen) {
    if (!cfg || !q || !rhs || q == rhs) {
        set_err(err, errlen, "null or aliased argument");
        return HERMES_ERR_ARG;
    }
    if (!supported(*cfg)) {
        set_err(err, errlen, "unsupported configuration");
        return HERMES_ERR_CONFIG;
    }
    const hermes_config& c = *cfg;
    KernelSet K = kernels_for(c);

    // the grid descriptor of one box (the geometry hermes_create builds)
    Box b;
    std::memset(&b, 0, sizeof(b));
    b.n[0] = c.nx; b.n[1] = c.ny; b.n[2] = c.nz;
    long long nface[3];
    for (int k = 0; k < 6; ++k) b.bc[k] = c.bc[k];
    for (int d = 0; d < 3; ++d)
        b.nfp[d] = (c.bc[2 * d] == HERMES_BC_PERIODIC && c.bc[2 * d + 1] == HERMES_BC_PERIODIC) ? b.n[d] : b.n[d] + 1;
    b.ncell = (long long)c.nx * c.ny * c.nz;
    const double L[3] = {c.lx, c.ly, c.lz};
    for (int d = 0; d < 3; ++d) {
        long long f = 1;
        for (int e = 0; e < 3; ++e) f *= (e == d ? b.nfp[e] : b.n[e]);
        nface[d] = f;
        b.di[d] = (double)b.n[d] / L[d];
    }
    b.cflm = c.cflm > 0 ? c.cflm : (c.iquad == 3 ? 0.08 : 0.14);
    b.seed = c.seed;
    b.fbase[0] = 0;
    b.fbase[1] = nface[0] * NQ * K.nf;
    b.fbase[2] = b.fbase[1] + nface[1] * NQ * K.nf;
    const unsigned long long flux_bytes =
        (unsigned long long)(b.fbase[2] + nface[2] * NQ * K.nf) * (unsigned long long)K.elem_size;
    if (flux_bytes > (unsigned long long)HERMES_NOALLOC_SCRATCH_BYTES) {
        char msg[256];
        std::snprintf(msg, sizeof(msg),
                      "grid needs %llu bytes of face-flux scratch; the static maximum is %llu bytes",
                      flux_bytes, (unsigned long long)HERMES_NOALLOC_SCRATCH_BYTES);
        set_err(err, errlen, msg);
        return HERMES_ERR_SHAPE;
    }

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { set_err(err, errlen, cudaGetErrorString(e)); return HERMES_ERR_CUDA; }
    DevAddrs* A = nullptr;
    int rc = device_addrs(dev, &A, err, errlen);
    if (rc) return rc;
    e = K.prepare();
    if (e != cudaSuccess) { set_err(err, errlen, cudaGetErrorString(e)); return HERMES_ERR_CUDA; }

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_noalloc_records<<<1, 1, 0, s>>>(b);
    e = cudaGetLastError();
    if (e != cudaSuccess) { set_err(err, errlen, cudaGetErrorString(e)); return HERMES_ERR_CUDA; }

    Phys ph{};
    ph.aindex = c.aindex; ph.aindm1 = c.aindex - 1.0; ph.rh_floor = c.rh_floor; ph.T_floor = c.T_floor;
    ph.P_floor = c.T_floor * c.rh_floor; ph.rh_mult = c.rh_mult; ph.coll = c.coll; ph.colvis = c.colvis;
    ph.P_1 = c.P_1; ph.P_base = c.P_base; ph.eta_sd = c.eta_sd; ph.zeta_sd = c.zeta_sd;
    ph.body_force = c.body_force; ph.ivis = c.ivis; ph.ieos = c.ieos; ph.ihllc = c.ihllc;
    ph.llns = c.llns ? 1 : 0;
    phys_finish(ph);
    Geom G{};
    G.boxes = A->box;
    G.nbox = 1;
    G.ncell = b.ncell;
    for (int d = 0; d < 3; ++d) G.nface[d] = nface[d];

    if (apply_limiter && (c.ieos == 1 || c.ieos == 2)) K.limit(q, G, ph, s);
    FaceArgs fa{G, ph, A->step, 0u};
    for (int d = 0; d < 3; ++d) K.face(d, q, A->scratch, fa, s);
    CellArgs ca{G, ph, A->state, A->step, A->flags, 0u, MODE_RHS, COMB_NONE, 0};
    K.cell(q, nullptr, rhs, A->scratch, ca, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) { set_err(err, errlen, cudaGetErrorString(e)); return HERMES_ERR_CUDA; }
    return HERMES_OK;
}

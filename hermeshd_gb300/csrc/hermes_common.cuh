// hermes_common.cuh -- shared device types and compile-time helpers of the
// GB300 DG step.  Layout of one grid ("box"): the reference's Fortran
// Q(nx,ny,nz,nQ,nbasis), i.e. element (b, v, cell) at (b*NQ + v)*ncell + cell
// with cell = i + nx*(j + ny*k).  An ensemble stores its boxes back to back.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>
#include <utility>

#include "dg_tables_gen.cuh"

namespace hermes {

constexpr int NQ = 11;  // params.f90:47
enum Var { RH = 0, MX, MY, MZ, EN, PXX, PYY, PZZ, PXY, PXZ, PYZ };
enum Bc { BC_PERIODIC = 0, BC_OUTFLOW = 1, BC_WALL = 2, BC_NOSLIP = 3, BC_INFLOW = 4 };

// device error flags (plain stores; read by the host after a step)
enum Flag { FLAG_NONFINITE = 1 };

// compile-time loop: f(std::integral_constant<int, i>) for i in [0, N)
template <class F, int... I>
__device__ __forceinline__ void sfor_impl(F&& f, std::integer_sequence<int, I...>) {
    (f(std::integral_constant<int, I>{}), ...);
}
template <int N, class F>
__device__ __forceinline__ void sfor(F&& f) {
    sfor_impl(f, std::make_integer_sequence<int, N>{});
}

// run-time loop over [0, N) whose body is still instantiated per index
// (compile-time tables stay constant); iterations are not interleaved by the
// scheduler, which bounds register pressure for large bodies
template <int N, class F>
__device__ __forceinline__ void sfor_seq(F&& f) {
#pragma unroll 1
    for (int i = 0; i < N; ++i) {
        sfor<N>([&](auto I) {
            if (i == decltype(I)::value) f(I);
        });
    }
}

// block barrier reached by different warps from different call sites (the
// two thread groups of k_cell run different instantiations of one phase):
// the non-.aligned barrier, which each warp reaches uniformly
__device__ __forceinline__ void block_sync_split() { asm volatile("barrier.sync 0;" ::: "memory"); }

// physics constants (params.f90 / input.f90), identical for every box
struct Phys {
    double aindex, aindm1, rh_floor, T_floor, P_floor, rh_mult;
    double coll, colvis, P_1, P_base;
    double eta_sd, zeta_sd, body_force;
    double inflow_u, inflow_rho, inflow_p, inflow_ly;   // parabolic x-low inflow (BC_INFLOW)
    int ivis, ieos, ihllc, llns;
    double roe_cp;   // aindex / aindm1 (the Roe enthalpy's factor), set by phys_finish
    // the same constants rounded to float once on the host (phys_finish): the
    // FP32 kernels read these instead of converting a double per use, a
    // conversion that runs on the FP64 pipe
    float f_aindex, f_aindm1, f_rh_floor, f_T_floor, f_P_floor, f_rh_mult, f_coll, f_colvis, f_P_1, f_P_base;
    float f_eta_sd, f_zeta_sd, f_body_force, f_roe_cp;
};

// fill the float copies (round to nearest, as a conversion on the device would)
inline void phys_finish(Phys& p) {
    p.f_aindex = (float)p.aindex; p.f_aindm1 = (float)p.aindm1; p.f_rh_floor = (float)p.rh_floor;
    p.f_T_floor = (float)p.T_floor; p.f_P_floor = (float)p.P_floor; p.f_rh_mult = (float)p.rh_mult;
    p.f_coll = (float)p.coll; p.f_colvis = (float)p.colvis; p.f_P_1 = (float)p.P_1; p.f_P_base = (float)p.P_base;
    p.f_eta_sd = (float)p.eta_sd; p.f_zeta_sd = (float)p.zeta_sd; p.f_body_force = (float)p.body_force;
    p.roe_cp = p.aindex / p.aindm1;
    p.f_roe_cp = (float)p.roe_cp;
}

// a physics constant in the arithmetic type T: the float copy for T = float,
// the double converted to T otherwise
template <class T>
__host__ __device__ __forceinline__ T phys_const(double d, float f) {
    if constexpr (std::is_same<T, float>::value) return f;
    else return T(d);
}
#define PHC(T, ph, name) (::hermes::phys_const<T>((ph).name, (ph).f_##name))

// one grid of the run (one realisation of an ensemble)
struct Box {
    int n[3];                 // nx, ny, nz
    int nfp[3];               // face planes per direction: n (both ends periodic) or n+1
    int bc[6];                // xlo, xhi, ylo, yhi, zlo, zhi
    int pad_;
    long long ncell;          // nx*ny*nz
    long long cell0;          // first cell of this box in the global cell numbering
    long long q0;             // first element of this box in a Q buffer
    long long face0[3];       // first face of this box in the global face numbering, per direction
    long long fbase[3];       // first element of this box's face-flux array, per direction
    double di[3];             // dxi, dyi, dzi
    double cflm;
    unsigned long long seed;  // Philox key of the stochastic stress
};

// per-box device scalars
struct BoxState {
    double dt, t;
    unsigned long long vmag_bits;  // max wave speed (bit pattern of a non-negative double)
    double cs_last;                // sound speed of the last cell (hermeshd.f90:174)
};

// box of a global index: boxes sorted by `first`, binary search
template <class Getter>
__device__ __forceinline__ int find_box(const Box* __restrict__ boxes, int nbox, long long idx, Getter first) {
    int lo = 0, hi = nbox - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (first(boxes[mid]) <= idx) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <class T>
__device__ __forceinline__ T tfma(T a, T b, T c) { return fma(a, b, c); }

// Programmatic dependent launch: a step kernel launched with the
// programmatic-serialisation attribute may start while the kernel before it
// in the stream finishes.  It waits for that kernel's completion and memory
// (griddepcontrol.wait) before its first global memory access, and lets the
// kernel after it start launching (griddepcontrol.launch_dependents), which
// overlaps each launch with the previous kernel's tail.  Without the
// attribute both instructions do nothing.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// launch a step kernel, with the programmatic-serialisation attribute when
// pdl is set (the kernel then begins with pdl_enter); errors are left for
// cudaGetLastError, as with <<<>>>
template <class... KArgs, class... Args>
inline void launch_k(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                     Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    (void)cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

}  // namespace hermes

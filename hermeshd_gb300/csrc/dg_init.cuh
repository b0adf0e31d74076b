// dg_init.cuh -- initial states of set_ic (initialcon.f90:20-361) built on the
// device, one thread per cell of every box, so a run's set-up never leaves
// the GPU.  Only the cell averages (basis function 1) are set, as in the
// reference; every other coefficient is written zero.
//   icid 0  hydro_jet (:79-114), its random kick from Philox-4x32-10 with
//           counter (cell_lo, cell_hi, JET_TAG, 0) and key = seed instead of
//           Fortran's unseeded random_number
//   icid 1  isentropic vortex, version 0 (:128-183)
//   icid 2  isentropic vortex, version 1
//   icid 3  Sod shock tube, version 0 (:190-235): high state where xc <= 0
//   icid 4  Sod shock tube, version 1: high state where xc + yc <= 0
//   icid 5-7  poiseuille_flow / pipe_cylinder_2d (:244-361): fluid at rest
// Cell centres follow params.f90:212-227 with the domain centred at the
// origin: xc = -lx/2 + (i + 1/2)/dxi, dxi = nx/lx.
#pragma once

#include "dg_physics.cuh"

namespace hermes {

constexpr int INIT_TPB = 256;
constexpr uint32_t JET_TAG = 0x4A455400u;

struct InitArgs {
    const Box* boxes;
    const double* len;        // lx, ly, lz per box
    int nbox;
    long long ncell;
    int nb;                   // basis functions per variable
    int icid;
    double aindex, rh_floor, T_floor, P_base;
    unsigned long long seed;
};

// the top 53 bits of the first two words of one Philox block, in [0, 1)
__device__ __forceinline__ double philox_u53(unsigned long long seed, unsigned long long site, uint32_t tag) {
    uint32_t c[4] = {(uint32_t)site, (uint32_t)(site >> 32), tag, 0u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const unsigned long long m = ((unsigned long long)c[0] << 21) | (unsigned long long)(c[1] >> 11);
    return (double)m * (1.0 / 9007199254740992.0);
}

template <class T>
__global__ void __launch_bounds__(INIT_TPB) k_init(T* __restrict__ Q, InitArgs a) {
    const long long gc = (long long)blockIdx.x * INIT_TPB + threadIdx.x;
    if (gc >= a.ncell) return;
    const int bx = find_box(a.boxes, a.nbox, gc, [](const Box& b) { return b.cell0; });
    const Box& B = a.boxes[bx];
    const long long le = gc - B.cell0, nc = B.ncell;
    const int i = (int)(le % B.n[0]), j = (int)((le / B.n[0]) % B.n[1]);
    const double lx = a.len[3 * bx], ly = a.len[3 * bx + 1];
    const double xc = -(lx / 2.0) + (i + 0.5) * (1.0 / B.di[0]);
    const double yc = -(ly / 2.0) + (j + 0.5) * (1.0 / B.di[1]);
    const double g = a.aindex, aindm1 = g - 1.0;
    // initialcon.f90:35-37: floor density and energy everywhere first
    double rh = a.rh_floor, mx = 0.0, my = 0.0, mz = 0.0, en = a.T_floor * a.rh_floor / aindm1;
    auto hydro = [&](double dn, double vx, double vy, double vz, double pr) {
        rh = dn;
        mx = dn * vx;
        my = dn * vy;
        mz = dn * vz;
        en = pr / aindm1 + 0.5 * dn * (vx * vx + vy * vy + vz * vz);
    };
    const double pi = 3.14159265358979323846;
    if (a.icid == 0) {
        const double dn = 1.0, te = a.T_floor, pr = te * dn, beta = 1.0, beta2 = 0.005;
        const double rnum = philox_u53(a.seed, (unsigned long long)le, JET_TAG) - 0.5;
        const double ch = cosh(20.0 * yc / (ly / 2.0));
        const double smx = beta * dn / ch, smy = beta2 * rnum / (ch * ch);
        rh = dn;
        mx = smx;
        my = smy;
        mz = 0.0;
        en = pr / aindm1 + 0.5 * (smx * smx + smy * smy + 0.0 * 0.0) / dn;
    } else if (a.icid == 1 || a.icid == 2) {
        const double beta = 5.0, vx_amb = 1.0, vy_amb = a.icid == 1 ? 0.0 : 1.0, Rgsqi = a.icid == 1 ? 1.0 : 0.5;
        const double r2 = xc * xc + yc * yc;
        const double e1 = exp(Rgsqi * (1.0 - r2));
        const double dvx = -yc * beta / (2.0 * pi) * e1;
        const double dvy = xc * beta / (2.0 * pi) * e1;
        const double dT = -(aindm1 * (beta * beta)) / (16.0 * Rgsqi * g * (pi * pi)) * exp(2.0 * Rgsqi * (1.0 - r2));
        const double te = 1.0 + dT;
        const double dn = pow(te, 1.0 / aindm1);
        hydro(dn, vx_amb + dvx, vy_amb + dvy, 0.0, pow(dn, g));
    } else if (a.icid == 3 || a.icid == 4) {
        const double s = xc + (a.icid == 4 ? yc : 0.0);
        if (s <= 0.0) hydro(1.0, 0.0, 0.0, 0.0, 1.0 * a.P_base);
        else hydro(0.125, 0.0, 0.0, 0.0, 0.1 * a.P_base);
    } else {
        hydro(1.0, 0.0, 0.0, 0.0, a.T_floor * 1.0);
    }
    T* Qb = Q + B.q0;
    const double avg[5] = {rh, mx, my, mz, en};
    for (int b = 0; b < a.nb; ++b)
        for (int v = 0; v < NQ; ++v) Qb[(long long)(b * NQ + v) * nc + le] = (b == 0 && v < 5) ? (T)avg[v] : T(0);
}

cudaError_t init_launch(int precision, void* Q, const InitArgs& a, cudaStream_t s);

}  // namespace hermes

namespace hermes {

// ---------------------------------------------------------------------------
// Conservation sums in FP64 for any precision of the state: per box, the
// integrals of rho, m_x, m_y, m_z and E (cell averages times the cell
// volume).  Each box is cut into chunks of CONS_CHUNK cells; one block sums a
// chunk in a fixed order, then one block per box sums its chunks in order, so
// the result does not depend on scheduling.
// ---------------------------------------------------------------------------
constexpr int CONS_TPB = 256;
constexpr int CONS_CHUNK = 8192;

struct ConsArgs {
    const Box* boxes;
    const int* chunk_box;       // box of each chunk
    const int* box_chunk0;      // first chunk of each box (nbox + 1 entries)
    double* partial;            // 5 per chunk
    double* out;                // 5 per box
    int nchunk;
};

template <class T>
__global__ void __launch_bounds__(CONS_TPB) k_cons_partial(const T* __restrict__ Q, ConsArgs a) {
    __shared__ double red[5][CONS_TPB];
    const int ch = blockIdx.x;
    const int bx = a.chunk_box[ch];
    const Box& B = a.boxes[bx];
    const long long first = (long long)(ch - a.box_chunk0[bx]) * CONS_CHUNK;
    const long long last = first + CONS_CHUNK < B.ncell ? first + CONS_CHUNK : B.ncell;
    const T* Qb = Q + B.q0;
    double s[5] = {0, 0, 0, 0, 0};
    for (long long c = first + threadIdx.x; c < last; c += CONS_TPB)
#pragma unroll
        for (int v = 0; v < 5; ++v) s[v] += (double)Qb[(long long)v * B.ncell + c];
#pragma unroll
    for (int v = 0; v < 5; ++v) red[v][threadIdx.x] = s[v];
    __syncthreads();
    for (int k = CONS_TPB / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k)
#pragma unroll
            for (int v = 0; v < 5; ++v) red[v][threadIdx.x] += red[v][threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x < 5) a.partial[5 * ch + threadIdx.x] = red[threadIdx.x][0];
}

cudaError_t cons_launch(int precision, const void* Q, const ConsArgs& a, int nbox, cudaStream_t s);

}  // namespace hermes

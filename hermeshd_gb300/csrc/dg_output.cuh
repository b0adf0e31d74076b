// dg_output.cuh -- derived fields of the VTK output (output.f90:14-317), on
// the device.
//
// k_derived evaluates the modal state at nvtk^3 sub-points per cell (the
// reference's bfvtk tables, basis_funcs.f90:88-200: point s of nvtk along an
// axis at (2s+1-nvtk)/nvtk in reference coordinates) and writes the selected
// VTK variables as float32 (the reference's R4P output), one array per
// variable, sub-cells x fastest (the VTK cell order of output.f90):
//   0 Density rho*n0            1 Log density log(rho*n0)/log(10)
//   2-4 Velocity v0*m/rho       5 Temperature P*te0/(rho*eV_per_K)
//   6 Internal energy density   7 Total energy density
//   8 Entropy density P*rho^-(gamma-1)   9 Pressure
//   10-12 Isotropic stress pxx, pyy, pzz
//   13 Vorticity -2 (d_x v_y - d_y v_x) dxi / t0, the derivatives taken in
//      reference coordinates (the d/dxi of bfvtk_dx, scaled by dxi alone as
//      the reference does)
// P = (gamma-1)(E - rho v^2/2) for every equation of state, as in the
// reference's output.
#pragma once

#include "dg_kernels.cuh"

namespace hermes {

constexpr int DV_N = 14;
constexpr int DERIVED_TPB = 128;

struct DerivedArgs {
    Geom G;                       // one box
    double aindex;
    double n0, v0, t0, te0, eV_per_K;
    int nvtk;
    unsigned mask;                // bit v set: variable v is written
    int slot[DV_N];               // output array of variable v (its rank among the selected)
};

__device__ __forceinline__ double leg(int deg, double s) {
    return deg == 0 ? 1.0 : deg == 1 ? s : 1.5 * (s * s) - 0.5;
}
__device__ __forceinline__ double dleg(int deg, double s) {
    return deg == 0 ? 0.0 : deg == 1 ? 1.0 : 3.0 * s;
}

template <class T, class TB>
__global__ void __launch_bounds__(DERIVED_TPB) k_derived(const T* __restrict__ Q, float* __restrict__ out,
                                                         DerivedArgs a) {
    constexpr int NB = TB::NB;
    const Box& B = a.G.boxes[0];
    const int nv = a.nvtk;
    const long long nnx = (long long)B.n[0] * nv, nny = (long long)B.n[1] * nv, nnz = (long long)B.n[2] * nv;
    const long long total = nnx * nny * nnz;
    const long long l = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= total) return;
    const long long i = l % nnx, j = (l / nnx) % nny, k = l / (nnx * nny);
    const long long cell = i / nv + B.n[0] * (j / nv + (long long)B.n[1] * (k / nv));
    // sub-point coordinate (2s + 1 - nvtk)/nvtk: -1/2, 1/2; -2/3, 0, 2/3; ... as the reference's xgrid
    const double x = (double)(2 * (i % nv) + 1 - nv) / nv;
    const double y = (double)(2 * (j % nv) + 1 - nv) / nv;
    const double z = (double)(2 * (k % nv) + 1 - nv) / nv;
    const long long nc = B.ncell;
    // point values of rh..en and the diagonal stresses; x and y derivatives of rh, mx, my
    constexpr int NVAL = 8;
    constexpr int VAR[NVAL] = {RH, MX, MY, MZ, EN, PXX, PYY, PZZ};
    double u[NVAL], drx = 0.0, dry = 0.0, dmyx = 0.0, dmxy = 0.0;
#pragma unroll
    for (int m = 0; m < NVAL; ++m) u[m] = 0.0;
    sfor<NB>([&](auto bb) {
        constexpr int b = decltype(bb)::value;
        constexpr int ex = TB::DEG(b, 0), ey = TB::DEG(b, 1), ez = TB::DEG(b, 2);
        const double lx = leg(ex, x), ly = leg(ey, y), lz = leg(ez, z);
        const double phi = (lx * ly) * lz;
        const double px = (dleg(ex, x) * ly) * lz, py = (lx * dleg(ey, y)) * lz;
#pragma unroll
        for (int m = 0; m < NVAL; ++m) u[m] = fma(phi, (double)Q[(long long)(b * NQ + VAR[m]) * nc + cell], u[m]);
        const double qr = (double)Q[(long long)(b * NQ + RH) * nc + cell];
        drx = fma(px, qr, drx);
        dry = fma(py, qr, dry);
        dmyx = fma(px, (double)Q[(long long)(b * NQ + MY) * nc + cell], dmyx);
        dmxy = fma(py, (double)Q[(long long)(b * NQ + MX) * nc + cell], dmxy);
    });
    const double dn = u[0], dni = 1.0 / dn;
    const double vx = u[1] * dni, vy = u[2] * dni, vz = u[3] * dni;
    const double U = u[4] - 0.5 * dn * (vx * vx + vy * vy + vz * vz);
    const double P = (a.aindex - 1.0) * U;
    const unsigned mask = a.mask;
    auto put = [&](int v, double val) { out[(long long)a.slot[v] * total + l] = (float)val; };
    // quotients by rho taken as products with 1/rho (one FP64 rounding apart,
    // below the float32 output's resolution); every variable only when asked for
    if (mask & (1u << 0)) put(0, dn * a.n0);
    // log and pow in FP32: the output is float32, and the FP64 forms cost more
    // than the rest of the kernel (single-precision results are within 2 ulps)
    if (mask & (1u << 1)) put(1, (double)(logf((float)(dn * a.n0)) * 0.43429448190325182f));
    if (mask & (1u << 2)) put(2, a.v0 * vx);
    if (mask & (1u << 3)) put(3, a.v0 * vy);
    if (mask & (1u << 4)) put(4, a.v0 * vz);
    if (mask & (1u << 5)) put(5, P * a.te0 * dni / a.eV_per_K);
    if (mask & (1u << 6)) put(6, U);
    if (mask & (1u << 7)) put(7, u[4]);
    if (mask & (1u << 8)) put(8, (double)((float)P * powf((float)dni, (float)(a.aindex - 1.0))));
    if (mask & (1u << 9)) put(9, P);
    if (mask & (1u << 10)) put(10, u[5]);
    if (mask & (1u << 11)) put(11, u[6]);
    if (mask & (1u << 12)) put(12, u[7]);
    if (mask & (1u << 13)) {
        const double dni2 = dni * dni;
        const double dxvy = (dn * dmyx - u[2] * drx) * dni2;
        const double dyvx = (dn * dmxy - u[1] * dry) * dni2;
        put(13, -2.0 * (dxvy - dyvx) * B.di[0] / a.t0);
    }
}

template <class T, int NB, int NQD>
cudaError_t derived_launch(const void* Q, float* out, const DerivedArgs& a, cudaStream_t s) {
    using TB = hermes_tab::Tab<NB, NQD>;
    const long long total = (long long)a.G.ncell * a.nvtk * a.nvtk * a.nvtk;
    if (total <= 0) return cudaSuccess;
    k_derived<T, TB><<<(unsigned)((total + DERIVED_TPB - 1) / DERIVED_TPB), DERIVED_TPB, 0, s>>>(
        static_cast<const T*>(Q), out, a);
    return cudaGetLastError();
}

using DerivedFn = cudaError_t (*)(const void*, float*, const DerivedArgs&, cudaStream_t);
bool derived_launcher(int precision, int nb, DerivedFn* out);

}  // namespace hermes

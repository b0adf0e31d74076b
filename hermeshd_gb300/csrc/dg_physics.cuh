// dg_physics.cuh -- point-wise physics of the DG step: the 5/10-moment point
// flux (flux.f90:23-193), the HLLC Riemann solver (flux.f90:466-647), the
// freezing speed (flux.f90:1029-1072) and the stochastic stress
// (random.f90:106-145, with a counter-based Philox generator).
//
// Everything here is evaluated at one quadrature point by one thread.  T is
// the arithmetic type of the bulk path (double, or float for the FP32 path).
#pragma once

#include "hermes_common.cuh"

namespace hermes {

// ---------------------------------------------------------------------------
// Philox-4x32-10 (Salmon et al., SC'11).  Counter scheme:
//   key = seed, counter = (site, pt | kind<<8 | sub<<12 | stage<<16, step_lo, step_hi)
// kind: 0..2 face call in x/y/z, 3..5 interior call in x/y/z.  The stress of
// a point needs six independent normals: random.f90:124-141 symmetrises a
// 3x3 matrix of nine iid N(0,1) values, whose three diagonal entries and three
// scaled sums sqrt(1/2) (G_ij + G_ji) are six iid N(0,1) values -- drawn here
// directly.  Two blocks (sub 0, 1) give eight 32-bit words, one uniform each;
// three Box-Muller pairs of the first six give the six normals.
// ---------------------------------------------------------------------------
struct NoiseCtr {
    unsigned long long step;
    unsigned stage;
};

__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// one Box-Muller pair from two 32-bit words; every rounding explicit (no
// contraction into FMAs), so the numbers do not depend on the kernel the
// generator is inlined into
template <class T>
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, T& z0, T& z1) {
    if constexpr (std::is_same<T, double>::value) {
        // 32-bit uniforms in (0,1): (w + 1/2) 2^-32
        const double u1 = __dmul_rn(__dadd_rn((double)a, 0.5), 1.0 / 4294967296.0);
        const double u2 = __dmul_rn(__dadd_rn((double)b, 0.5), 1.0 / 4294967296.0);
        double r = sqrt(__dmul_rn(-2.0, log(u1))), s, co;
        sincos(__dmul_rn(6.283185307179586476925286766559, u2), &s, &co);
        z0 = __dmul_rn(r, co); z1 = __dmul_rn(r, s);
    } else {
        // the top 24 bits of the same words; the hardware log2 and sin/cos
        // (absolute error ~2^-21 on (-pi, pi)), with the angle moved to
        // (-pi, pi) by cos(t - pi) = -cos t, sin(t - pi) = -sin t
        const float u1 = __fmul_rn(__fadd_rn((float)(a >> 8), 0.5f), 1.0f / 16777216.0f);
        const float u2 = __fmul_rn(__fadd_rn((float)(b >> 8), 0.5f), 1.0f / 16777216.0f);
        float r = sqrtf(__fmul_rn(-2.0f, __logf(u1))), s, co;
        __sincosf(__fmul_rn(6.2831853071795864769f, __fsub_rn(u2, 0.5f)), &s, &co);
        z0 = -__fmul_rn(r, co); z1 = -__fmul_rn(r, s);
    }
}

// G = {xx, yy, zz, xy, xz, yz}: the diagonal and the symmetrised off-diagonal normals
template <class T>
__device__ __forceinline__ void normals6(unsigned long long seed, NoiseCtr nc, unsigned kind, unsigned long long site,
                                         unsigned pt, T G[6]) {
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    uint32_t w[8];
#pragma unroll
    for (int sub = 0; sub < 2; ++sub) {
        uint32_t* c = w + 4 * sub;
        c[0] = (uint32_t)site;
        c[1] = (pt & 0xFFu) | ((kind & 0xFu) << 8) | (((unsigned)sub & 0xFu) << 12) | ((nc.stage & 0xFFFFu) << 16);
        c[2] = (uint32_t)nc.step;
        c[3] = (uint32_t)(nc.step >> 32);
        philox4x32_10(c, k0, k1);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) box_muller<T>(w[2 * k], w[2 * k + 1], G[2 * k], G[2 * k + 1]);
}

// random.f90:106-145: S = eta (sym G - tr G/3 I) + zeta tr G I, the
// amplitudes already carrying 1/sqrt(dV dt).  S = {xx, yy, zz, xy, xz, yz}.
template <class T>
__device__ __forceinline__ void random_stress_amp(T eta, T zeta, unsigned long long seed, NoiseCtr nc, unsigned kind,
                                                  unsigned long long site, unsigned pt, T S[6]) {
    T G[6];
    normals6<T>(seed, nc, kind, site, pt, G);
    // explicit roundings, as in box_muller: the same numbers in every kernel
    auto add = [](T x, T y) { if constexpr (std::is_same<T, double>::value) return __dadd_rn(x, y); else return __fadd_rn(x, y); };
    auto sub = [](T x, T y) { if constexpr (std::is_same<T, double>::value) return __dsub_rn(x, y); else return __fsub_rn(x, y); };
    auto mul = [](T x, T y) { if constexpr (std::is_same<T, double>::value) return __dmul_rn(x, y); else return __fmul_rn(x, y); };
    T trG = add(add(G[0], G[1]), G[2]), trGd3 = trG / T(3), trGz = mul(zeta, trG);
    S[0] = add(mul(eta, sub(G[0], trGd3)), trGz);
    S[1] = add(mul(eta, sub(G[1], trGd3)), trGz);
    S[2] = add(mul(eta, sub(G[2], trGd3)), trGz);
    S[3] = mul(eta, G[3]);
    S[4] = mul(eta, G[4]);
    S[5] = mul(eta, G[5]);
}

template <class T>
__device__ __forceinline__ void random_stress(const Phys& ph, unsigned long long seed, NoiseCtr nc, unsigned kind,
                                              unsigned long long site, unsigned pt, T S[6]) {
    random_stress_amp<T>(PHC(T, ph, eta_sd), PHC(T, ph, zeta_sd), seed, nc, kind, site, pt, S);
}

// ---------------------------------------------------------------------------
// flux.f90:23-193 flux_calc_pnts_r at one point, direction DIR (0 x, 1 y, 2 z)
// ---------------------------------------------------------------------------
template <class T>
struct Prim {
    T dn, dni, vx, vy, vz, P, P_10;
    T Pig;   // ideal-gas pressure before the Tait term and the floor (HLLC's p)
};

template <class T>
__device__ __forceinline__ Prim<T> primitives(const Phys& ph, const T q[NQ]) {
    Prim<T> w;
    w.dn = q[RH];
    w.dni = T(1) / w.dn;
    w.vx = q[MX] * w.dni;
    w.vy = q[MY] * w.dni;
    w.vz = q[MZ] * w.dni;
    T smsq = q[MX] * q[MX] + q[MY] * q[MY] + q[MZ] * q[MZ];
    w.P = PHC(T, ph, aindm1) * (q[EN] - T(0.5) * w.dni * smsq);
    w.Pig = w.P;
    if (ph.ieos == 2) w.P = PHC(T, ph, P_1) * (pow(w.dn, T(7.2)) - T(1)) + PHC(T, ph, P_base) + w.P;
    const T Pf = PHC(T, ph, P_floor);
    if (w.P < Pf) w.P = Pf;
    // the 10-moment pressure enters only the ivis 2/3 fluxes (flux.f90:91-95)
    if (ph.ivis >= 2) {
        w.P_10 = T(1.0 / 3.0) * (q[PXX] + q[PYY] + q[PZZ] - w.dni * smsq);
        if (w.P_10 < Pf) w.P_10 = Pf;
    } else {
        w.P_10 = T(0);
    }
    return w;
}

// S = {Sxx, Syy, Szz, Sxy, Sxz, Syz} (zero without noise)
template <class T, int DIR>
__device__ __forceinline__ void point_flux(const Phys& ph, const T q[NQ], const Prim<T>& w, const T S[6], T f[NQ]) {
    const T colvis = PHC(T, ph, colvis);
    const T c2d3cv = T(2.0 / 3.0) * colvis, c4d3cv = T(4.0 / 3.0) * colvis;
    const T M_x = q[MX], M_y = q[MY], M_z = q[MZ], Ener = q[EN];
    const T P_xx = q[PXX], P_yy = q[PYY], P_zz = q[PZZ], P_xy = q[PXY], P_xz = q[PXZ], P_yz = q[PYZ];
    const T vx = w.vx, vy = w.vy, vz = w.vz, P = w.P, P_10 = w.P_10, P_5 = w.P;
    const T Sxx = S[0], Syy = S[1], Szz = S[2], Sxy = S[3], Sxz = S[4], Syz = S[5];
    const bool tenm = (ph.ivis >= 2);   // ivis 2 and the Grad closure (ivis 3)
    if constexpr (DIR == 0) {
        f[RH] = M_x;
        if (!tenm) {
            f[MX] = M_x * vx + P + P_xx - Sxx;
            f[MY] = M_y * vx + P_xy - Sxy;
            f[MZ] = M_z * vx + P_xz - Sxz;
        } else {
            f[MX] = P_xx - P_10 + P_5;
            f[MY] = P_xy;
            f[MZ] = P_xz;
        }
        f[EN] = (Ener + P) * vx + (P_xx - Sxx) * vx + (P_xy - Sxy) * vy + (P_xz - Sxz) * vz;
        if (ph.ivis == 3) f[EN] = (Ener + P) * vx;   // Grad closure: ten_moment.f90:969
        if (!tenm) {
            f[PXX] = c4d3cv * vx; f[PYY] = -c2d3cv * vx; f[PZZ] = -c2d3cv * vx;
            f[PXY] = colvis * vy; f[PXZ] = colvis * vz; f[PYZ] = T(0);
        } else {
            f[PXX] = vx * (T(3) * P_xx - T(2) * vx * M_x);
            f[PYY] = T(2) * vy * (P_xy - vy * M_x) + vx * P_yy;
            f[PZZ] = T(2) * vz * (P_xz - vz * M_x) + vx * P_zz;
            f[PXY] = T(2) * vx * (P_xy - vy * M_x) + vy * P_xx;
            f[PXZ] = T(2) * vx * (P_xz - vz * M_x) + vz * P_xx;
            f[PYZ] = vx * P_yz + vy * P_xz + vz * P_xy - T(2) * vy * vz * M_x;
        }
    } else if constexpr (DIR == 1) {
        f[RH] = M_y;
        if (!tenm) {
            f[MX] = M_x * vy + P_xy - Sxy;
            f[MY] = M_y * vy + P + P_yy - Syy;
            f[MZ] = M_z * vy + P_yz - Syz;
        } else {
            f[MX] = P_xy;
            f[MY] = P_yy - P_10 + P_5;
            f[MZ] = P_yz;
        }
        f[EN] = (Ener + P) * vy + (P_yy - Syy) * vy + (P_xy - Sxy) * vx + (P_yz - Syz) * vz;
        if (ph.ivis == 3) f[EN] = (Ener + P) * vy;   // Grad closure: ten_moment.f90:969
        if (!tenm) {
            f[PXX] = -c2d3cv * vy; f[PYY] = c4d3cv * vy; f[PZZ] = -c2d3cv * vy;
            f[PXY] = colvis * vx; f[PXZ] = T(0); f[PYZ] = colvis * vz;
        } else {
            f[PXX] = T(2) * vx * (P_xy - vx * M_y) + vy * P_xx;
            f[PYY] = vy * (T(3) * P_yy - T(2) * vy * M_y);
            f[PZZ] = T(2) * vz * (P_yz - vz * M_y) + vy * P_zz;
            f[PXY] = T(2) * vy * (P_xy - vx * M_y) + vx * P_yy;
            f[PXZ] = vx * P_yz + vy * P_xz + vz * P_xy - T(2) * vx * vz * M_y;
            f[PYZ] = T(2) * vy * (P_yz - vz * M_y) + vz * P_yy;
        }
    } else {
        f[RH] = M_z;
        if (!tenm) {
            f[MX] = M_x * vz + P_xz - Sxz;
            f[MY] = M_y * vz + P_yz - Syz;
            f[MZ] = M_z * vz + P + P_zz - Szz;
        } else {
            f[MX] = P_xz;
            f[MY] = P_yz;
            f[MZ] = P_zz - P_10 + P_5;
        }
        f[EN] = (Ener + P) * vz + (P_zz - Szz) * vz + (P_xz - Sxz) * vx + (P_yz - Syz) * vy;
        if (ph.ivis == 3) f[EN] = (Ener + P) * vz;   // Grad closure: ten_moment.f90:969
        if (!tenm) {
            f[PXX] = -c2d3cv * vz; f[PYY] = -c2d3cv * vz; f[PZZ] = c4d3cv * vz;
            f[PXY] = T(0); f[PXZ] = colvis * vx; f[PYZ] = colvis * vy;
        } else {
            f[PXX] = T(2) * vx * (P_xz - vx * M_z) + vz * P_xx;
            f[PYY] = T(2) * vy * (P_yz - vy * M_z) + vz * P_yy;
            f[PZZ] = vz * (T(3) * P_zz - T(2) * vz * M_z);
            f[PXY] = vx * P_yz + vy * P_xz + vz * P_xy - T(2) * vx * vy * M_z;
            f[PXZ] = T(2) * vz * (P_xz - vx * M_z) + vx * P_zz;
            f[PYZ] = T(2) * vz * (P_yz - vy * M_z) + vy * P_zz;
        }
    }
}

// sources.f90:51-69: the ivis 2 point source of the stresses,
// coll rho (v_i v_j - delta_ij |v|^2 / 3), S = {xx, yy, zz, xy, xz, yz}
// (shared by the cell kernel and the adjoint's dual passes)
template <class T>
__device__ __forceinline__ void ten_moment_source(const Phys& ph, const Prim<T>& w, T s[6]) {
    const T vx2 = w.vx * w.vx, vy2 = w.vy * w.vy, vz2 = w.vz * w.vz;
    const T colldn = PHC(T, ph, coll) * w.dn, c1d3 = T(1.0 / 3.0);
    s[0] = colldn * (T(2) * vx2 - vy2 - vz2) * c1d3;
    s[1] = colldn * (T(2) * vy2 - vz2 - vx2) * c1d3;
    s[2] = colldn * (T(2) * vz2 - vx2 - vy2) * c1d3;
    s[3] = colldn * w.vx * w.vy;
    s[4] = colldn * w.vx * w.vz;
    s[5] = colldn * w.vy * w.vz;
}

// flux.f90:1029-1072 cfcal: freezing speed |v_d| + c
template <class T, int DIR>
__device__ __forceinline__ T cfcal(const Phys& ph, const T q[NQ]) {
    T dn = q[RH], dni = T(1) / dn;
    T vx = q[MX] * dni, vy = q[MY] * dni, vz = q[MZ] * dni;
    T P;
    if (ph.ivis == 0 || ph.ivis == 1) P = PHC(T, ph, aindm1) * (q[EN] - T(0.5) * dn * (vx * vx + vy * vy + vz * vz));
    else P = T(1.0 / 3.0) * (q[PXX] + q[PYY] + q[PZZ] - dn * (vx * vx + vy * vy + vz * vz));
    T cs;
    if (ph.ieos == 1) cs = sqrt(PHC(T, ph, aindex) * P * dni);
    else cs = sqrt(T(7.2) * PHC(T, ph, P_1) * pow(dn, T(6.2)));
    T vd = DIR == 0 ? vx : DIR == 1 ? vy : vz;
    return fabs(vd) + cs;
}

// ---------------------------------------------------------------------------
// flux.f90:466-647 flux_hllc (ibatten = 0) at one face point.  qL/qR, fL/fR:
// left/right states and point fluxes.  rho_i_last: 1/rho of the last point of
// the call (the reference's ieos-2 branch uses it for every point,
// flux.f90:533-534,570-571); unused for ieos 1.  Writes rh..en of F.
// ---------------------------------------------------------------------------
template <class T, int DIR>
__device__ __forceinline__ void hllc(const Phys& ph, const T qL[NQ], const T qR[NQ], const T fL[NQ], const T fR[NQ],
                                     const Prim<T>& PL, const Prim<T>& PR, T rho_i_last, T F[NQ]) {
    // PL, PR: the primitives of the two states (primitives()).  The velocities
    // are theirs; p is the unfloored ideal-gas pressure, which flux.f90:525
    // forms as aindm1 (E - rho |v|^2 / 2): here aindm1 (E - |m|^2 / rho / 2),
    // equal to rounding
    constexpr int IPAR = DIR == 0 ? MX : DIR == 1 ? MY : MZ;
    constexpr int IP1 = DIR == 0 ? MY : DIR == 1 ? MZ : MX;
    constexpr int IP2 = DIR == 0 ? MZ : DIR == 1 ? MX : MY;
    const T aindex = PHC(T, ph, aindex);
    const T dniL = PL.dni, dniR = PR.dni;
    const T rhoL = qL[RH], rhoR = qR[RH];
    const T uL = DIR == 0 ? PL.vx : DIR == 1 ? PL.vy : PL.vz;
    const T uR = DIR == 0 ? PR.vx : DIR == 1 ? PR.vy : PR.vz;
    T pL = PL.Pig;
    T pR = PR.Pig;
    T cL, cR;
    if (ph.ieos == 2) {
        pL = PHC(T, ph, P_1) * (pow(rhoL, T(7.2)) - T(1)) + PHC(T, ph, P_base) + pL;
        pR = PHC(T, ph, P_1) * (pow(rhoR, T(7.2)) - T(1)) + PHC(T, ph, P_base) + pR;
        cL = sqrt(T(7.2) * PHC(T, ph, P_1) * pow(rhoL, T(6.2)) + pL * rho_i_last);
        cR = sqrt(T(7.2) * PHC(T, ph, P_1) * pow(rhoR, T(6.2)) + pR * rho_i_last);
    } else {
        // sqrt(aindex*p/rho) of flux.f90:537-538, with the division taken as
        // a product with 1/rho (one rounding apart; two divisions fewer)
        cL = sqrt(aindex * pL * dniL);
        cR = sqrt(aindex * pR * dniR);
    }
    // S_L = min(lambda_M(Q_l), lambda_M(Q_r)); S_R = max(lambda_P(Q_r), lambda_P(Q_l))
    const T sL = fmin(uL - cL, uR - cR);
    const T sR = fmax(uR + cR, uL + cL);
    T sm_num = rhoR * uR * (sR - uR) - rhoL * uL * (sL - uL);
    sm_num = sm_num + pL - pR;
    T sm_den = rhoR * (sR - uR) - rhoL * (sL - uL);
    if (sm_den == T(0)) sm_den = PHC(T, ph, rh_floor);
    const T sM = sm_num / sm_den;
    const T pstar = rhoL * (uL - sL) * (uL - sM) + pL;
    // flux.f90:623-643: the last true condition wins
    int which = -1;
    if (sL > T(0)) which = 0;
    if (sL <= T(0) && T(0) < sM) which = 1;
    if (sM <= T(0) && T(0) <= sR) which = 2;
    if (sR < T(0)) which = 3;
    T out[5];
    if (which == 0 || which == 3) {
        const T* ff = which == 0 ? fL : fR;
        out[0] = ff[RH]; out[1] = ff[IPAR]; out[2] = ff[IP1]; out[3] = ff[IP2]; out[4] = ff[EN];
    } else if (which >= 0) {
        const bool left = which == 1;
        const T* q = left ? qL : qR;
        const T* ff = left ? fL : fR;
        const T s = left ? sL : sR, rho = left ? rhoL : rhoR, u = left ? uL : uR, p = left ? pL : pR;
        T den = s - sM;
        if (den == T(0)) den = PHC(T, ph, rh_floor);
        const T slrm_i = T(1) / den;
        const T sq = s - u;
        const T Q0 = rho * sq * slrm_i;
        const T Q1 = (sq * q[IPAR] + pstar - p) * slrm_i;
        const T Q2 = sq * q[IP1] * slrm_i;
        const T Q3 = sq * q[IP2] * slrm_i;
        const T Q4 = (sq * q[EN] - p * u + pstar * sM) * slrm_i;
        out[0] = ff[RH] + s * (Q0 - q[RH]);
        out[1] = ff[IPAR] + s * (Q1 - q[IPAR]);
        out[2] = ff[IP1] + s * (Q2 - q[IP1]);
        out[3] = ff[IP2] + s * (Q3 - q[IP2]);
        out[4] = ff[EN] + s * (Q4 - q[EN]);
    } else {
        const T nan = T(NAN);
        out[0] = out[1] = out[2] = out[3] = out[4] = nan;
    }
    F[RH] = out[0]; F[IPAR] = out[1]; F[IP1] = out[2]; F[IP2] = out[3]; F[EN] = out[4];
}


// ---------------------------------------------------------------------------
// Roe solver of the monolithic 10-moment code
// (src/ces/10_moment/dg_3D_hydro_lqc_SEAN.f90:1614-1789) at one face point.
// Returns false (kroe = 0: keep the central/LLF flux) when the Roe sound
// speed squared is <= 0; otherwise writes rh..en of F.  The Roe enthalpy
// keeps the reference's factor 1/2 on its pressure term (:1676).
// ---------------------------------------------------------------------------
template <class T, int DIR>
__device__ __forceinline__ bool roe(const Phys& ph, const T qL[NQ], const T qR[NQ], const T fL[NQ], const T fR[NQ],
                                    T F[NQ]) {
    constexpr int IP = DIR == 0 ? MX : DIR == 1 ? MY : MZ;
    constexpr int I1 = DIR == 0 ? MY : DIR == 1 ? MZ : MX;
    constexpr int I2 = DIR == 0 ? MZ : DIR == 1 ? MX : MY;
    const T aindm1 = PHC(T, ph, aindm1), cp = PHC(T, ph, roe_cp);
    T skr[2], swr[2][4];
#pragma unroll
    for (int j9 = 0; j9 < 2; ++j9) {
        const T* q = j9 == 0 ? qL : qR;
        const T dnii = T(1) / q[RH];
        const T v0 = q[IP] * dnii, v1 = q[I1] * dnii, v2 = q[I2] * dnii;
        const T vsq = v0 * v0 + v1 * v1 + v2 * v2;
        const T Pri = aindm1 * (q[EN] - T(0.5) * q[RH] * vsq);
        skr[j9] = sqrt(q[RH]);
        swr[j9][0] = skr[j9] * v0;
        swr[j9][1] = skr[j9] * v1;
        swr[j9][2] = skr[j9] * v2;
        swr[j9][3] = T(0.5) * skr[j9] * (vsq + cp * Pri / q[RH]);
    }
    const T Qri = T(1) / qL[RH];
    const T delrho = qR[RH] * Qri - T(1);
    const T dele = (qR[EN] - qL[EN]) * Qri;
    const T dm1 = (qR[IP] - qL[IP]) * Qri, dm2 = (qR[I1] - qL[I1]) * Qri, dm3 = (qR[I2] - qL[I2]) * Qri;
    const T dsk = T(0.5) * (skr[1] + skr[0]);
    const T vc0 = T(0.5) * (swr[1][0] + swr[0][0]) / dsk;
    const T vc1 = T(0.5) * (swr[1][1] + swr[0][1]) / dsk;
    const T vc2 = T(0.5) * (swr[1][2] + swr[0][2]) / dsk;
    const T hc = T(0.5) * (swr[1][3] + swr[0][3]) / dsk;
    const T vcsq = vc0 * vc0 + vc1 * vc1 + vc2 * vc2;
    const T asq = aindm1 * (hc - T(0.5) * vcsq);
    if (!(asq > T(0))) return false;
    const T sc9 = sqrt(asq);
    const T l0 = fabs(vc0 - sc9), l1 = fabs(vc0 + sc9), l2 = fabs(vc0);
    const T ea2i = aindm1 / asq;
    const T vcdel = vc0 * dm1 + vc1 * dm2 + vc2 * dm3 - dele;
    const T a9e = T(0.5) * ea2i * (T(0.5) * vcsq * delrho - vcdel);
    const T sk9 = T(0.5) * (dm1 - vc0 * delrho) / sc9;
    const T w0 = (a9e - sk9) * l0, w1 = (a9e + sk9) * l1, w2 = ea2i * ((hc - vcsq) * delrho + vcdel) * l2;
    const T w3 = (dm2 - vc1 * delrho) * l2, w4 = (dm3 - vc2 * delrho) * l2;
    // dF = sum_j w_j evec(:, j), scaled by rho_L
    const T d0 = (w0 + w1 + w2) * qL[RH];
    const T d1 = (w0 * (hc - sc9 * vc0) + w1 * (hc + sc9 * vc0) + w2 * (T(0.5) * vcsq) + w3 * vc1 + w4 * vc2) * qL[RH];
    const T d2 = (w0 * (vc0 - sc9) + w1 * (vc0 + sc9) + w2 * vc0) * qL[RH];
    const T d3 = ((w0 + w1 + w2) * vc1 + w3) * qL[RH];
    const T d4 = ((w0 + w1 + w2) * vc2 + w4) * qL[RH];
    F[RH] = T(0.5) * (fL[RH] + fR[RH] - d0);
    F[EN] = T(0.5) * (fL[EN] + fR[EN] - d1);
    F[IP] = T(0.5) * (fL[IP] + fR[IP] - d2);
    F[I1] = T(0.5) * (fL[I1] + fR[I1] - d3);
    F[I2] = T(0.5) * (fL[I2] + fR[I2] - d4);
    return true;
}

}  // namespace hermes

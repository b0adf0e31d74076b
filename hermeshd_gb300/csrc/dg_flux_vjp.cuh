// dg_flux_vjp.cuh -- hand-derived reverse-mode vector-Jacobian product of the
// numerical face flux of face_flux_fn (FP64; ivis 0/1, ieos 1, no stochastic
// stress): given lamF = dL/dF at one face point, lamL = (dF/dqL)^T lamF and
// lamR = (dF/dqR)^T lamF.  One primal sweep keeps the intermediates, one
// reverse sweep applies the chain rule term by term; branches (HLLC wave
// selection, Roe |lambda| and its fallback, the pressure floor, min/max)
// follow their primal outcome, as the dual-number passes do.
//
//   primitives + point flux   flux.f90:23-193 (restated in dg_physics.cuh)
//   central average           flux.f90:256-262 (ivis < 2: no LLF term)
//   HLLC                      flux.f90:466-647 (ibatten 0)
//   Roe                       src/ces/10_moment/dg_3D_hydro_lqc_SEAN.f90:1614-1789
#pragma once

#include "dg_kernels.cuh"

namespace hermes {

// primal quantities of one side kept for the reverse sweep
struct SideRev {
    double dni, v[3], smsq, P;
    bool clamped;
};

// primitives of dg_physics.cuh (ieos 1): dni, velocities, pressure (floored)
__device__ __forceinline__ SideRev side_primal(const Phys& ph, const double q[NQ]) {
    SideRev s;
    s.dni = 1.0 / q[RH];
    s.v[0] = q[MX] * s.dni;
    s.v[1] = q[MY] * s.dni;
    s.v[2] = q[MZ] * s.dni;
    s.smsq = q[MX] * q[MX] + q[MY] * q[MY] + q[MZ] * q[MZ];
    s.P = ph.aindm1 * (q[EN] - 0.5 * s.dni * s.smsq);
    s.clamped = s.P < ph.P_floor;
    if (s.clamped) s.P = ph.P_floor;
    return s;
}

// reverse of point_flux<DIR> (ivis 0/1) then of the primitives:
// lf = dL/df, accumulates dL/dq into lq
template <int DIR>
__device__ __forceinline__ void point_flux_rev(const Phys& ph, const double q[NQ], const SideRev& s, const double lf[NQ],
                                               double lq[NQ]) {
    constexpr int MD = MX + DIR;   // momentum along DIR
    // stress component (DIR, i) of the momentum rows
    constexpr int PS[3][3] = {{PXX, PXY, PXZ}, {PXY, PYY, PYZ}, {PXZ, PYZ, PZZ}};
    const double vd = s.v[DIR];
    double lv[3] = {0.0, 0.0, 0.0}, lP = 0.0;
    // f[RH] = M_d
    lq[MD] += lf[RH];
    // f[M_i] = M_i v_d + (i == d) P + P_{d i}
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        lq[MX + i] += lf[MX + i] * vd;
        lv[DIR] += lf[MX + i] * q[MX + i];
        lq[PS[DIR][i]] += lf[MX + i];
    }
    lP += lf[MD];
    // f[E] = (E + P) v_d + sum_i P_{d i} v_i
    lq[EN] += lf[EN] * vd;
    lP += lf[EN] * vd;
    lv[DIR] += lf[EN] * (q[EN] + s.P);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        lq[PS[DIR][i]] += lf[EN] * s.v[i];
        lv[i] += lf[EN] * q[PS[DIR][i]];
    }
    // stress rows: colvis times (4/3, -2/3, -2/3) v_d on the diagonal, colvis v_i off it
    const double cv = ph.colvis, c4 = (4.0 / 3.0) * cv, c2 = (2.0 / 3.0) * cv;
    if (DIR == 0) {
        lv[0] += c4 * lf[PXX] - c2 * lf[PYY] - c2 * lf[PZZ];
        lv[1] += cv * lf[PXY];
        lv[2] += cv * lf[PXZ];
    } else if (DIR == 1) {
        lv[1] += -c2 * lf[PXX] + c4 * lf[PYY] - c2 * lf[PZZ];
        lv[0] += cv * lf[PXY];
        lv[2] += cv * lf[PYZ];
    } else {
        lv[2] += -c2 * lf[PXX] - c2 * lf[PYY] + c4 * lf[PZZ];
        lv[0] += cv * lf[PXZ];
        lv[1] += cv * lf[PYZ];
    }
    // primitives: P = aindm1 (E - dni smsq / 2) unless floored; v_i = M_i dni; dni = 1/rho
    double ldni = 0.0;
    if (!s.clamped) {
        lq[EN] += ph.aindm1 * lP;
        ldni += -0.5 * ph.aindm1 * s.smsq * lP;
#pragma unroll
        for (int i = 0; i < 3; ++i) lq[MX + i] += -ph.aindm1 * s.dni * q[MX + i] * lP;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        lq[MX + i] += lv[i] * s.dni;
        ldni += lv[i] * q[MX + i];
    }
    lq[RH] += -s.dni * s.dni * ldni;
}

// reverse of hllc<double, DIR> (ieos 1): lo = dL/d out[rh..en rows];
// accumulates into lqL, lqR (state) and lfL, lfR (point fluxes, rows rh..en)
template <int DIR>
__device__ __forceinline__ void hllc_rev(const Phys& ph, const double qL[NQ], const double qR[NQ], const double fL[NQ],
                                         const double fR[NQ], double dniL, double dniR, const double lF[NQ],
                                         double lqL[NQ], double lqR[NQ], double lfL[NQ], double lfR[NQ]) {
    constexpr int IPAR = DIR == 0 ? MX : DIR == 1 ? MY : MZ;
    constexpr int IP1 = DIR == 0 ? MY : DIR == 1 ? MZ : MX;
    constexpr int IP2 = DIR == 0 ? MZ : DIR == 1 ? MX : MY;
    constexpr int ROW[5] = {RH, IPAR, IP1, IP2, EN};
    const double aindex = ph.aindex, aindm1 = ph.aindm1;
    // ---- primal
    const double rhoL = qL[RH], rhoR = qR[RH];
    const double uL = qL[IPAR] * dniL, vL = qL[IP1] * dniL, wL = qL[IP2] * dniL;
    const double uR = qR[IPAR] * dniR, vR = qR[IP1] * dniR, wR = qR[IP2] * dniR;
    const double kL = uL * uL + vL * vL + wL * wL, kR = uR * uR + vR * vR + wR * wR;
    const double pL = aindm1 * (qL[EN] - 0.5 * rhoL * kL);
    const double pR = aindm1 * (qR[EN] - 0.5 * rhoR * kR);
    const double cL = sqrt(aindex * pL * dniL), cR = sqrt(aindex * pR * dniR);
    const double aL = uL - cL, aR = uR - cR, bR = uR + cR, bL = uL + cL;
    const bool sLfromR = aR < aL, sRfromL = bL > bR;
    const double sL = sLfromR ? aR : aL, sR = sRfromL ? bL : bR;
    double sm_num = rhoR * uR * (sR - uR) - rhoL * uL * (sL - uL);
    sm_num = sm_num + pL - pR;
    double sm_den = rhoR * (sR - uR) - rhoL * (sL - uL);
    const bool den0 = sm_den == 0.0;
    if (den0) sm_den = ph.rh_floor;
    const double sM = sm_num / sm_den;
    const double pstar = rhoL * (uL - sL) * (uL - sM) + pL;
    int which = -1;
    if (sL > 0.0) which = 0;
    if (sL <= 0.0 && 0.0 < sM) which = 1;
    if (sM <= 0.0 && 0.0 <= sR) which = 2;
    if (sR < 0.0) which = 3;
    // ---- reverse
    double lrhoL = 0, lrhoR = 0, luL = 0, luR = 0, lvL = 0, lvR = 0, lwL = 0, lwR = 0;
    double lpL = 0, lpR = 0, lsL = 0, lsR = 0, lsM = 0, lpstar = 0;
    if (which == 0 || which == 3) {
        double* lf = which == 0 ? lfL : lfR;
#pragma unroll
        for (int k = 0; k < 5; ++k) lf[ROW[k]] += lF[ROW[k]];
    } else if (which >= 0) {
        const bool left = which == 1;
        const double* q = left ? qL : qR;
        double* lq = left ? lqL : lqR;
        double* lf = left ? lfL : lfR;
        const double s = left ? sL : sR, rho = left ? rhoL : rhoR, u = left ? uL : uR, p = left ? pL : pR;
        double den = s - sM;
        const bool dfl = den == 0.0;
        if (dfl) den = ph.rh_floor;
        const double slrm = 1.0 / den, sq = s - u;
        const double Qs[5] = {rho * sq * slrm, (sq * q[IPAR] + pstar - p) * slrm, sq * q[IP1] * slrm,
                              sq * q[IP2] * slrm, (sq * q[EN] - p * u + pstar * sM) * slrm};
        double ls = 0, lsq = 0, lslrm = 0, lrho = 0, lu = 0, lp = 0;
        double lQ[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            lf[ROW[k]] += lF[ROW[k]];
            ls += lF[ROW[k]] * (Qs[k] - q[ROW[k]]);
            lQ[k] = s * lF[ROW[k]];
            lq[ROW[k]] += -s * lF[ROW[k]];
        }
        // Q0 = rho sq slrm
        lrho += lQ[0] * sq * slrm; lsq += lQ[0] * rho * slrm; lslrm += lQ[0] * rho * sq;
        // Q1 = (sq q_par + pstar - p) slrm
        lsq += lQ[1] * q[IPAR] * slrm; lq[IPAR] += lQ[1] * sq * slrm; lpstar += lQ[1] * slrm; lp -= lQ[1] * slrm;
        lslrm += lQ[1] * (sq * q[IPAR] + pstar - p);
        // Q2, Q3 = sq q_t slrm
        lsq += lQ[2] * q[IP1] * slrm; lq[IP1] += lQ[2] * sq * slrm; lslrm += lQ[2] * sq * q[IP1];
        lsq += lQ[3] * q[IP2] * slrm; lq[IP2] += lQ[3] * sq * slrm; lslrm += lQ[3] * sq * q[IP2];
        // Q4 = (sq E - p u + pstar sM) slrm
        lsq += lQ[4] * q[EN] * slrm; lq[EN] += lQ[4] * sq * slrm; lp -= lQ[4] * u * slrm; lu -= lQ[4] * p * slrm;
        lpstar += lQ[4] * sM * slrm; lsM += lQ[4] * pstar * slrm;
        lslrm += lQ[4] * (sq * q[EN] - p * u + pstar * sM);
        // slrm = 1/den, den = s - sM (a floored den is a constant)
        if (!dfl) {
            const double lden = -slrm * slrm * lslrm;
            ls += lden;
            lsM -= lden;
        }
        // sq = s - u
        ls += lsq;
        lu -= lsq;
        if (left) { lsL += ls; lrhoL += lrho; luL += lu; lpL += lp; }
        else { lsR += ls; lrhoR += lrho; luR += lu; lpR += lp; }
    }
    // pstar = rhoL (uL - sL)(uL - sM) + pL
    lrhoL += lpstar * (uL - sL) * (uL - sM);
    luL += lpstar * rhoL * ((uL - sM) + (uL - sL));
    lsL -= lpstar * rhoL * (uL - sM);
    lsM -= lpstar * rhoL * (uL - sL);
    lpL += lpstar;
    // sM = sm_num / sm_den
    const double lnum = lsM / sm_den, lden = den0 ? 0.0 : -lsM * sM / sm_den;
    // sm_num = rhoR uR (sR - uR) - rhoL uL (sL - uL) + pL - pR
    lrhoR += lnum * uR * (sR - uR);
    luR += lnum * rhoR * ((sR - uR) - uR);
    lsR += lnum * rhoR * uR;
    lrhoL -= lnum * uL * (sL - uL);
    luL -= lnum * rhoL * ((sL - uL) - uL);
    lsL -= lnum * rhoL * uL;
    lpL += lnum;
    lpR -= lnum;
    // sm_den = rhoR (sR - uR) - rhoL (sL - uL)
    lrhoR += lden * (sR - uR);
    lsR += lden * rhoR;
    luR -= lden * rhoR;
    lrhoL -= lden * (sL - uL);
    lsL -= lden * rhoL;
    luL += lden * rhoL;
    // sL = min(uL - cL, uR - cR), sR = max(uR + cR, uL + cL)
    double lcL = 0, lcR = 0;
    if (sLfromR) { luR += lsL; lcR -= lsL; } else { luL += lsL; lcL -= lsL; }
    if (sRfromL) { luL += lsR; lcL += lsR; } else { luR += lsR; lcR += lsR; }
    // c = sqrt(aindex p dni)
    double ldniL = 0, ldniR = 0;
    if (cL > 0.0) { lpL += lcL * aindex * dniL / (2.0 * cL); ldniL += lcL * aindex * pL / (2.0 * cL); }
    if (cR > 0.0) { lpR += lcR * aindex * dniR / (2.0 * cR); ldniR += lcR * aindex * pR / (2.0 * cR); }
    // p = aindm1 (E - rho k / 2), k = u^2 + v^2 + w^2
    lqL[EN] += aindm1 * lpL;
    lrhoL -= 0.5 * aindm1 * kL * lpL;
    luL -= aindm1 * rhoL * uL * lpL; lvL -= aindm1 * rhoL * vL * lpL; lwL -= aindm1 * rhoL * wL * lpL;
    lqR[EN] += aindm1 * lpR;
    lrhoR -= 0.5 * aindm1 * kR * lpR;
    luR -= aindm1 * rhoR * uR * lpR; lvR -= aindm1 * rhoR * vR * lpR; lwR -= aindm1 * rhoR * wR * lpR;
    // u = q_par dni, v = q_1 dni, w = q_2 dni; dni = 1/rho; rho = q_rh
    lqL[IPAR] += luL * dniL; lqL[IP1] += lvL * dniL; lqL[IP2] += lwL * dniL;
    ldniL += luL * qL[IPAR] + lvL * qL[IP1] + lwL * qL[IP2];
    lqR[IPAR] += luR * dniR; lqR[IP1] += lvR * dniR; lqR[IP2] += lwR * dniR;
    ldniR += luR * qR[IPAR] + lvR * qR[IP1] + lwR * qR[IP2];
    lqL[RH] += lrhoL - dniL * dniL * ldniL;
    lqR[RH] += lrhoR - dniR * dniR * ldniR;
}

// reverse of roe<double, DIR>: returns false (nothing accumulated) where the
// primal falls back to the central flux
template <int DIR>
__device__ __forceinline__ bool roe_rev(const Phys& ph, const double qL[NQ], const double qR[NQ], const double lF[NQ],
                                        double lqL[NQ], double lqR[NQ], double lfL[NQ], double lfR[NQ]) {
    constexpr int IP = DIR == 0 ? MX : DIR == 1 ? MY : MZ;
    constexpr int I1 = DIR == 0 ? MY : DIR == 1 ? MZ : MX;
    constexpr int I2 = DIR == 0 ? MZ : DIR == 1 ? MX : MY;
    const double aindm1 = ph.aindm1, cp = ph.aindex / ph.aindm1;
    // ---- primal (as roe<>)
    double dnii[2], vv[2][3], vsq[2], Pri[2], skr[2], swr[2][4];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const double* q = j == 0 ? qL : qR;
        dnii[j] = 1.0 / q[RH];
        vv[j][0] = q[IP] * dnii[j]; vv[j][1] = q[I1] * dnii[j]; vv[j][2] = q[I2] * dnii[j];
        vsq[j] = vv[j][0] * vv[j][0] + vv[j][1] * vv[j][1] + vv[j][2] * vv[j][2];
        Pri[j] = aindm1 * (q[EN] - 0.5 * q[RH] * vsq[j]);
        skr[j] = sqrt(q[RH]);
        swr[j][0] = skr[j] * vv[j][0]; swr[j][1] = skr[j] * vv[j][1]; swr[j][2] = skr[j] * vv[j][2];
        swr[j][3] = 0.5 * skr[j] * (vsq[j] + cp * Pri[j] / q[RH]);
    }
    const double Qri = 1.0 / qL[RH];
    const double delrho = qR[RH] * Qri - 1.0;
    const double dele = (qR[EN] - qL[EN]) * Qri;
    const double dm1 = (qR[IP] - qL[IP]) * Qri, dm2 = (qR[I1] - qL[I1]) * Qri, dm3 = (qR[I2] - qL[I2]) * Qri;
    const double dsk = 0.5 * (skr[1] + skr[0]);
    const double vc0 = 0.5 * (swr[1][0] + swr[0][0]) / dsk, vc1 = 0.5 * (swr[1][1] + swr[0][1]) / dsk;
    const double vc2 = 0.5 * (swr[1][2] + swr[0][2]) / dsk, hc = 0.5 * (swr[1][3] + swr[0][3]) / dsk;
    const double vcsq = vc0 * vc0 + vc1 * vc1 + vc2 * vc2;
    const double asq = aindm1 * (hc - 0.5 * vcsq);
    if (!(asq > 0.0)) return false;
    const double sc9 = sqrt(asq);
    const double x0 = vc0 - sc9, x1 = vc0 + sc9;
    const double l0 = fabs(x0), l1 = fabs(x1), l2 = fabs(vc0);
    const double ea2i = aindm1 / asq;
    const double vcdel = vc0 * dm1 + vc1 * dm2 + vc2 * dm3 - dele;
    const double a9e = 0.5 * ea2i * (0.5 * vcsq * delrho - vcdel);
    const double sk9 = 0.5 * (dm1 - vc0 * delrho) / sc9;
    const double A0 = a9e - sk9, A1 = a9e + sk9, A2 = ea2i * ((hc - vcsq) * delrho + vcdel);
    const double A3 = dm2 - vc1 * delrho, A4 = dm3 - vc2 * delrho;
    const double w0 = A0 * l0, w1 = A1 * l1, w2 = A2 * l2, w3 = A3 * l2, w4 = A4 * l2;
    const double W = w0 + w1 + w2, rL = qL[RH];
    const double e0 = W;
    const double e1 = w0 * (hc - sc9 * vc0) + w1 * (hc + sc9 * vc0) + w2 * (0.5 * vcsq) + w3 * vc1 + w4 * vc2;
    const double e2 = w0 * (vc0 - sc9) + w1 * (vc0 + sc9) + w2 * vc0;
    const double e3 = W * vc1 + w3, e4 = W * vc2 + w4;
    // ---- reverse.  F[row] = (fL + fR - d)/2 with d = e * rho_L
    const double lFr[5] = {lF[RH], lF[EN], lF[IP], lF[I1], lF[I2]};
    lfL[RH] += 0.5 * lF[RH]; lfR[RH] += 0.5 * lF[RH];
    lfL[EN] += 0.5 * lF[EN]; lfR[EN] += 0.5 * lF[EN];
    lfL[IP] += 0.5 * lF[IP]; lfR[IP] += 0.5 * lF[IP];
    lfL[I1] += 0.5 * lF[I1]; lfR[I1] += 0.5 * lF[I1];
    lfL[I2] += 0.5 * lF[I2]; lfR[I2] += 0.5 * lF[I2];
    const double ld[5] = {-0.5 * lFr[0], -0.5 * lFr[1], -0.5 * lFr[2], -0.5 * lFr[3], -0.5 * lFr[4]};
    const double e[5] = {e0, e1, e2, e3, e4};
    double lrL = 0.0, le[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) { lrL += ld[k] * e[k]; le[k] = ld[k] * rL; }
    double lw0 = 0, lw1 = 0, lw2 = 0, lw3 = 0, lw4 = 0, lhc = 0, lsc9 = 0, lvc0 = 0, lvc1 = 0, lvc2 = 0, lvcsq = 0;
    // e0 = W
    lw0 += le[0]; lw1 += le[0]; lw2 += le[0];
    // e1
    lw0 += le[1] * (hc - sc9 * vc0); lw1 += le[1] * (hc + sc9 * vc0); lw2 += le[1] * (0.5 * vcsq);
    lw3 += le[1] * vc1; lw4 += le[1] * vc2;
    lhc += le[1] * (w0 + w1);
    lsc9 += le[1] * (-w0 * vc0 + w1 * vc0);
    lvc0 += le[1] * (-w0 * sc9 + w1 * sc9);
    lvcsq += le[1] * 0.5 * w2;
    lvc1 += le[1] * w3; lvc2 += le[1] * w4;
    // e2
    lw0 += le[2] * (vc0 - sc9); lw1 += le[2] * (vc0 + sc9); lw2 += le[2] * vc0;
    lvc0 += le[2] * (w0 + w1 + w2); lsc9 += le[2] * (-w0 + w1);
    // e3 = W vc1 + w3, e4 = W vc2 + w4
    lw0 += le[3] * vc1 + le[4] * vc2; lw1 += le[3] * vc1 + le[4] * vc2; lw2 += le[3] * vc1 + le[4] * vc2;
    lvc1 += le[3] * W; lvc2 += le[4] * W;
    lw3 += le[3]; lw4 += le[4];
    // w = A * l
    double lA0 = lw0 * l0, lA1 = lw1 * l1, lA2 = lw2 * l2, lA3 = lw3 * l2, lA4 = lw4 * l2;
    const double ll0 = lw0 * A0, ll1 = lw1 * A1, ll2 = lw2 * A2 + lw3 * A3 + lw4 * A4;
    // l0 = |vc0 - sc9|, l1 = |vc0 + sc9|, l2 = |vc0| (the sign of the primal)
    const double g0 = x0 < 0.0 ? -ll0 : ll0, g1 = x1 < 0.0 ? -ll1 : ll1;
    lvc0 += g0 + g1 + (vc0 < 0.0 ? -ll2 : ll2);
    lsc9 += -g0 + g1;
    // A0 = a9e - sk9, A1 = a9e + sk9
    double la9e = lA0 + lA1, lsk9 = -lA0 + lA1;
    // A2 = ea2i ((hc - vcsq) delrho + vcdel)
    double lea2i = lA2 * ((hc - vcsq) * delrho + vcdel);
    lhc += lA2 * ea2i * delrho;
    lvcsq -= lA2 * ea2i * delrho;
    double ldelrho = lA2 * ea2i * (hc - vcsq);
    double lvcdel = lA2 * ea2i;
    // A3 = dm2 - vc1 delrho, A4 = dm3 - vc2 delrho
    double ldm1 = 0, ldm2 = lA3, ldm3 = lA4, ldele = 0;
    lvc1 -= lA3 * delrho; lvc2 -= lA4 * delrho;
    ldelrho -= lA3 * vc1 + lA4 * vc2;
    // sk9 = (dm1 - vc0 delrho) / (2 sc9)
    ldm1 += lsk9 * 0.5 / sc9;
    lvc0 -= lsk9 * 0.5 * delrho / sc9;
    ldelrho -= lsk9 * 0.5 * vc0 / sc9;
    lsc9 -= lsk9 * sk9 / sc9;
    // a9e = ea2i (vcsq delrho / 2 - vcdel) / 2
    lea2i += la9e * 0.5 * (0.5 * vcsq * delrho - vcdel);
    lvcsq += la9e * 0.25 * ea2i * delrho;
    ldelrho += la9e * 0.25 * ea2i * vcsq;
    lvcdel -= la9e * 0.5 * ea2i;
    // vcdel = vc . dm - dele
    lvc0 += lvcdel * dm1; lvc1 += lvcdel * dm2; lvc2 += lvcdel * dm3;
    ldm1 += lvcdel * vc0; ldm2 += lvcdel * vc1; ldm3 += lvcdel * vc2;
    ldele -= lvcdel;
    // ea2i = aindm1 / asq; sc9 = sqrt(asq)
    double lasq = -lea2i * ea2i / asq + lsc9 * 0.5 / sc9;
    // asq = aindm1 (hc - vcsq/2)
    lhc += lasq * aindm1;
    lvcsq -= lasq * 0.5 * aindm1;
    // vcsq = |vc|^2
    lvc0 += 2.0 * vc0 * lvcsq; lvc1 += 2.0 * vc1 * lvcsq; lvc2 += 2.0 * vc2 * lvcsq;
    // vc_k = (swr1_k + swr0_k) / (2 dsk), hc likewise with swr_3
    const double lvck[4] = {lvc0, lvc1, lvc2, lhc};
    const double vck[4] = {vc0, vc1, vc2, hc};
    double lswr[2][4], ldsk = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        lswr[0][k] = lswr[1][k] = 0.5 * lvck[k] / dsk;
        ldsk -= lvck[k] * vck[k] / dsk;
    }
    // dsk = (skr1 + skr0)/2
    double lskr[2] = {0.5 * ldsk, 0.5 * ldsk};
    // dm_k = (qR_k - qL_k) Qri, dele likewise, delrho = qR_rh Qri - 1; Qri = 1/qL_rh
    double lQri = ldm1 * (qR[IP] - qL[IP]) + ldm2 * (qR[I1] - qL[I1]) + ldm3 * (qR[I2] - qL[I2]) +
                  ldele * (qR[EN] - qL[EN]) + ldelrho * qR[RH];
    lqR[IP] += ldm1 * Qri; lqL[IP] -= ldm1 * Qri;
    lqR[I1] += ldm2 * Qri; lqL[I1] -= ldm2 * Qri;
    lqR[I2] += ldm3 * Qri; lqL[I2] -= ldm3 * Qri;
    lqR[EN] += ldele * Qri; lqL[EN] -= ldele * Qri;
    lqR[RH] += ldelrho * Qri;
    lqL[RH] += -Qri * Qri * lQri;
    lqL[RH] += lrL;
    // per side: swr_k = skr v_k (k < 3), swr_3 = skr (vsq + cp Pri / rho) / 2
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const double* q = j == 0 ? qL : qR;
        double* lq = j == 0 ? lqL : lqR;
        const double rinv = 1.0 / q[RH];
        double lv[3], lvsq, lPri, lrho = 0.0;
        lskr[j] += lswr[j][0] * vv[j][0] + lswr[j][1] * vv[j][1] + lswr[j][2] * vv[j][2];
#pragma unroll
        for (int k = 0; k < 3; ++k) lv[k] = lswr[j][k] * skr[j];
        const double h = vsq[j] + cp * Pri[j] * rinv;
        lskr[j] += lswr[j][3] * 0.5 * h;
        const double lh = lswr[j][3] * 0.5 * skr[j];
        lvsq = lh;
        lPri = lh * cp * rinv;
        lrho -= lh * cp * Pri[j] * rinv * rinv;
        // Pri = aindm1 (E - rho vsq / 2)
        lq[EN] += lPri * aindm1;
        lrho -= lPri * 0.5 * aindm1 * vsq[j];
        lvsq -= lPri * 0.5 * aindm1 * q[RH];
        // vsq = |v|^2
#pragma unroll
        for (int k = 0; k < 3; ++k) lv[k] += 2.0 * vv[j][k] * lvsq;
        // skr = sqrt(rho)
        lrho += lskr[j] * 0.5 / skr[j];
        // v_k = q_k dnii, dnii = 1/rho
        lq[IP] += lv[0] * dnii[j]; lq[I1] += lv[1] * dnii[j]; lq[I2] += lv[2] * dnii[j];
        const double ldn = lv[0] * q[IP] + lv[1] * q[I1] + lv[2] * q[I2];
        lrho += -dnii[j] * dnii[j] * ldn;
        lq[RH] += lrho;
    }
    return true;
}

// (dF/dqL)^T lF and (dF/dqR)^T lF of face_flux_fn<double, DIR> (ivis 0/1, ieos 1, no noise)
template <int DIR>
__device__ __forceinline__ void face_flux_vjp(const Phys& ph, const double qL[NQ], const double qR[NQ],
                                              const double lF[NQ], double lqL[NQ], double lqR[NQ]) {
    double fL[NQ], fR[NQ], lfL[NQ], lfR[NQ];
    const double S0[6] = {0, 0, 0, 0, 0, 0};
    const Prim<double> wL = primitives(ph, qL), wR = primitives(ph, qR);
    point_flux<double, DIR>(ph, qL, wL, S0, fL);
    point_flux<double, DIR>(ph, qR, wR, S0, fR);
#pragma unroll
    for (int v = 0; v < NQ; ++v) { lqL[v] = 0.0; lqR[v] = 0.0; lfL[v] = 0.5 * lF[v]; lfR[v] = 0.5 * lF[v]; }
    bool riemann = false;
    if (ph.ihllc == 2 || ph.ihllc == 1) {
        // rows rh..en come from the Riemann solver: undo their central share
        double lH[NQ];
#pragma unroll
        for (int v = 0; v < NQ; ++v) lH[v] = lF[v];
        double tL[NQ], tR[NQ];
#pragma unroll
        for (int v = 0; v < NQ; ++v) { tL[v] = 0.0; tR[v] = 0.0; }
        if (ph.ihllc == 2) {
            riemann = roe_rev<DIR>(ph, qL, qR, lH, lqL, lqR, tL, tR);
        } else {
            hllc_rev<DIR>(ph, qL, qR, fL, fR, wL.dni, wR.dni, lH, lqL, lqR, tL, tR);
            riemann = true;
        }
        if (riemann) {
#pragma unroll
            for (int v = RH; v <= EN; ++v) { lfL[v] = tL[v]; lfR[v] = tR[v]; }
        }
    }
    const SideRev sL = side_primal(ph, qL), sR = side_primal(ph, qR);
    point_flux_rev<DIR>(ph, qL, sL, lfL, lqL);
    point_flux_rev<DIR>(ph, qR, sR, lfR, lqR);
}

}  // namespace hermes

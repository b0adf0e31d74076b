// dg_adjoint.cuh -- vector-Jacobian products of the DG right-hand side and of
// one forward-Euler stage (FP64), the building blocks of the hand-written
// adjoint of the SSP-RK step.
//
// R(Q) = surface(F_face(traces(Q))) - volume(F_point(values(Q))) - source(Q)
// (flux.f90:932-1022, sources.f90:12-84).  The transpose of each linear map
// (traces, interior values, surface and volume quadrature) uses the same
// compile-time tables as the forward kernels; the point-wise nonlinear maps
// (numerical face flux, point fluxes, sources) contribute J^T lambda, by
// hand-derived reverse sweeps (dg_flux_vjp.cuh) or, as an independent check
// (HERMES_ADJOINT_DUAL=1), column by column with dual numbers run through the
// forward physics code.
//
//   k_face_adj  per face point: lambda of the face flux from mu of the two
//               cells that own the face, J^T of the numerical flux (one
//               hand-derived reverse sweep, dg_flux_vjp.cuh; or, as a check,
//               forward-mode dual passes), boundary ghost maps transposed;
//               writes the adjoint of both traces
//   k_cell_adj  per cell: gathers the trace adjoints, volume and source
//               transposes; writes nu = (dR/dQ)^T mu, or mu - dt*nu
//   k_limit_adj per cell: the positivity limiter's VJP (its active branch)
//
// Three ways to the point-wise Jacobians (MODE): ADJ_REV, the hand-derived
// reverse sweeps (ivis 0/1, ieos 1, no stochastic stress); ADJ_DUAL, their check path (dual passes
// for the hydro columns, the ivis 0/1 stress columns in closed form); ADJ_GEN,
// one dual pass per column of every variable through the forward physics,
// which covers whatever the forward computes: the 10-moment ivis 2 fluxes
// with the freezing-speed LLF flux and the nonlinear relaxation source
// (sources.f90:51-69), and the Tait equation of state (ieos 2) with the
// central or Roe flux.
//
// The stochastic stress is held fixed: ADJ_GEN redraws the forward kernels'
// values from the same Philox counters and passes them as constants.
//
// Scope: one grid, ivis 0, 1 or 2, ieos 1 or 2 (not ieos 2 with HLLC, whose
// every point uses 1/rho of the last point of the reference's call,
// flux.f90:533-534: a coupling across points).
#pragma once

#include "dg_dual.cuh"
#include "dg_flux_vjp.cuh"
#include "dg_launch.cuh"

namespace hermes {

// one side of a face: the cell and trace it comes from and the components a
// boundary ghost keeps (bit v set = kept); cell < 0: a zero ghost
struct TraceSrc {
    long long cell;
    int plus;
    unsigned mask;
};

template <class TB, int DIR, int P>
__device__ __forceinline__ double trace_of(const double* __restrict__ Qb, long long nc, const TraceSrc& s, int v) {
    if (s.cell < 0) return 0.0;
    double acc = 0.0;
    if (s.plus) {
        sfor<TB::NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            constexpr double c = ftab<TB, DIR, 1>(P, b);
            if constexpr (c != 0.0) acc = fma(c, Qb[(long long)(b * NQ + v) * nc + s.cell], acc);
        });
    } else {
        sfor<TB::NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            constexpr double c = ftab<TB, DIR, 0>(P, b);
            if constexpr (c != 0.0) acc = fma(c, Qb[(long long)(b * NQ + v) * nc + s.cell], acc);
        });
    }
    return ((s.mask >> v) & 1u) ? acc : 0.0;
}

template <class TB, int DIR, int P, int MODE>
__device__ __forceinline__ void face_adj_point(const double* __restrict__ Q, const double* __restrict__ mu,
                                               double* __restrict__ tadj, const AdjArgs& a, long long gf) {
    const Geom& G = a.G;
    const Phys& ph = a.ph;
    const Box& B = G.boxes[0];
    const long long lf = gf;
    const int n0 = B.n[0], n1 = B.n[1], n2 = B.n[2];
    const int ex = DIR == 0 ? B.nfp[0] : n0, ey = DIR == 1 ? B.nfp[1] : n1;
    const int i = (int)(lf % ex), j = (int)((lf / ex) % ey), k = (int)(lf / ((long long)ex * ey));
    const int n = B.n[DIR];
    const int s = DIR == 0 ? i : DIR == 1 ? j : k;
    const bool dedup = B.nfp[DIR] == n;
    const long long nc = B.ncell;
    auto cell_at = [&](int c) -> long long {
        int ci = DIR == 0 ? c : i, cj = DIR == 1 ? c : j, ck = DIR == 2 ? c : k;
        return (long long)ci + (long long)n0 * (cj + (long long)n1 * ck);
    };
    constexpr int MN = DIR == 0 ? MX : DIR == 1 ? MY : MZ;
    const unsigned all = (1u << NQ) - 1u;
    // sources of the two traces, boundary ghosts of boundary.f90:40-338
    TraceSrc L{-1, 1, all}, R{-1, 0, all};
    long long own_plus = -1, own_minus = -1;   // cells whose plus / minus face this is
    bool ghostL_from_R = false, ghostR_from_L = false;
    if (dedup || (s > 0 && s < n)) {
        const int lo = s > 0 ? s - 1 : n - 1;
        L = TraceSrc{cell_at(lo), 1, all};
        R = TraceSrc{cell_at(s), 0, all};
        own_plus = L.cell;
        own_minus = R.cell;
    } else if (s == 0) {
        R = TraceSrc{cell_at(0), 0, all};
        own_minus = R.cell;
        const int code = B.bc[2 * DIR];
        if (code != BC_PERIODIC) {
            unsigned m = all;
            if (code == BC_NOSLIP) m &= ~((1u << MX) | (1u << MY) | (1u << MZ));
            else if (code == BC_WALL) m &= ~(1u << MN);
            else if (code == BC_OUTFLOW) {
                double mmax = -INFINITY;
                sfor<TB::NF>([&](auto pp) {
                    mmax = fmax(mmax, trace_var<TB, DIR, 0, decltype(pp)::value, MN>(Q, nc, R.cell));
                });
                if (mmax > 0.0) m &= ~(1u << MN);
            }
            L = TraceSrc{R.cell, 0, m};
            ghostL_from_R = true;
        }
    } else {
        L = TraceSrc{cell_at(n - 1), 1, all};
        own_plus = L.cell;
        const int code = B.bc[2 * DIR + 1];
        // (a periodic high flag with a non-periodic low one is rejected by the host)
        if (code != BC_PERIODIC && !(code == BC_OUTFLOW && DIR == 0)) {
            unsigned m = all;
            if (code == BC_NOSLIP) m &= ~((1u << MX) | (1u << MY) | (1u << MZ));
            else if (code == BC_WALL) m &= ~(1u << MN);
            else if (code == BC_OUTFLOW) {
                double mmin = INFINITY;
                sfor<TB::NF>([&](auto pp) {
                    mmin = fmin(mmin, trace_var<TB, DIR, 1, decltype(pp)::value, MN>(Q, nc, L.cell));
                });
                if (mmin < 0.0) m &= ~(1u << MN);
            }
            R = TraceSrc{L.cell, 1, m};
            ghostR_from_L = true;
        }
    }
    double qL[NQ], qR[NQ];
#pragma unroll
    for (int v = 0; v < NQ; ++v) {
        qL[v] = trace_of<TB, DIR, P>(Q, nc, L, v);
        qR[v] = trace_of<TB, DIR, P>(Q, nc, R, v);
    }
    // adjoint of the stored face flux (F * di) from the surface assembly
    double lamF[NQ];
    const double di = B.di[DIR];
#pragma unroll
    for (int v = 0; v < NQ; ++v) {
        double sacc = 0.0;
        if (own_plus >= 0)
            sfor<TB::NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                constexpr double c = stab<TB, DIR, 1>(P, b);
                if constexpr (c != 0.0) sacc = fma(c, mu[(long long)(b * NQ + v) * nc + own_plus], sacc);
            });
        if (own_minus >= 0)
            sfor<TB::NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                constexpr double c = stab<TB, DIR, 0>(P, b);
                if constexpr (c != 0.0) sacc = fma(c, mu[(long long)(b * NQ + v) * nc + own_minus], sacc);
            });
        lamF[v] = di * sacc;
    }
    double lamL[NQ], lamR[NQ];
    if constexpr (MODE == ADJ_GEN) {
        // J^T lamF, one dual pass per column of each side's trace; the
        // stochastic stress of the face point (the forward face kernel's
        // draw: kind DIR, site lf, points P and P + NF) enters as a constant
        Dual SLd[6], SRd[6];
        if (ph.llns) {
            double SL[6], SR[6];
            const NoiseCtr nc{*a.nstep, a.nstage};
            random_stress<double>(ph, B.seed, nc, DIR, (unsigned long long)lf, P, SL);
            random_stress<double>(ph, B.seed, nc, DIR, (unsigned long long)lf, P + TB::NF, SR);
#pragma unroll
            for (int c = 0; c < 6; ++c) { SLd[c] = Dual(SL[c]); SRd[c] = Dual(SR[c]); }
        }
#pragma unroll 1
        for (int pass = 0; pass < 2 * NQ; ++pass) {
            const int side = pass / NQ, jv = pass % NQ;
            const TraceSrc& src = side == 0 ? L : R;
            double acc = 0.0;
            if (src.cell >= 0 && ((src.mask >> jv) & 1u)) {
                Dual dL[NQ], dR[NQ], F[NQ];
#pragma unroll
                for (int v = 0; v < NQ; ++v) {
                    dL[v] = Dual(qL[v], (side == 0 && v == jv) ? 1.0 : 0.0);
                    dR[v] = Dual(qR[v], (side == 1 && v == jv) ? 1.0 : 0.0);
                }
                face_flux_fn<Dual, DIR>(ph, dL, dR, SLd, SRd, Dual(0.0), F);
#pragma unroll
                for (int v = 0; v < NQ; ++v) acc = fma(lamF[v], F[v].d, acc);
            }
            (side == 0 ? lamL : lamR)[jv] = acc;
        }
    } else if constexpr (MODE == ADJ_REV) {
        // one reverse sweep through the numerical flux (dg_flux_vjp.cuh)
        face_flux_vjp<DIR>(ph, qL, qR, lamF, lamL, lamR);
        // a zero ghost or a ghost component forced to zero owns no trace
#pragma unroll
        for (int v = 0; v < NQ; ++v) {
            if (L.cell < 0 || !((L.mask >> v) & 1u)) lamL[v] = 0.0;
            if (R.cell < 0 || !((R.mask >> v) & 1u)) lamR[v] = 0.0;
        }
    } else {
        // J^T lamF.  Hydro columns (rh..en): one dual pass each.  Stress columns:
        // for ivis 0/1 the stresses enter only the point fluxes of the normal
        // direction, linearly (f[M_i] += P_{d i}, f[E] += P_{d i} v_i,
        // flux.f90:87-89), and every numerical flux takes f_L, f_R with weights
        // w_L + w_R = 1 (central and Roe 1/2 each; HLLC 1 on the side its wave
        // selection picks), so column P_{d i} of a side is w (lamF[M_i] + lamF[E] v_i).
        const Dual S0[6] = {Dual(0.0), Dual(0.0), Dual(0.0), Dual(0.0), Dual(0.0), Dual(0.0)};
        constexpr int PN[3] = {DIR == 0 ? PXX : DIR == 1 ? PXY : PXZ, DIR == 0 ? PXY : DIR == 1 ? PYY : PYZ,
                               DIR == 0 ? PXZ : DIR == 1 ? PYZ : PZZ};   // P_{d x}, P_{d y}, P_{d z}
        double wL = 0.0;
#pragma unroll 1
        for (int pass = -1; pass < 10; ++pass) {
            // pass -1: seed P_{d d} of the left trace, whose derivative in the
            // normal-momentum row is w_L; passes 0..9: hydro columns of L then R
            const int side = pass < 0 ? 0 : pass / 5, jv = pass < 0 ? PN[DIR] : pass % 5;
            const TraceSrc& src = side == 0 ? L : R;
            if (pass >= 0) {
                (side == 0 ? lamL : lamR)[jv] = 0.0;
                if (src.cell < 0 || !((src.mask >> jv) & 1u)) continue;
            }
            Dual dL[NQ], dR[NQ], F[NQ];
#pragma unroll
            for (int v = 0; v < NQ; ++v) {
                dL[v] = Dual(qL[v], (side == 0 && v == jv) ? 1.0 : 0.0);
                dR[v] = Dual(qR[v], (side == 1 && v == jv) ? 1.0 : 0.0);
            }
            face_flux_fn<Dual, DIR>(ph, dL, dR, S0, S0, Dual(0.0), F);
            if (pass < 0) {
                wL = F[MN].d;
                continue;
            }
            double acc = 0.0;
#pragma unroll
            for (int v = 0; v < NQ; ++v) acc = fma(lamF[v], F[v].d, acc);
            (side == 0 ? lamL : lamR)[jv] = acc;
        }
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const TraceSrc& src = side == 0 ? L : R;
            const double* qs = side == 0 ? qL : qR;
            double* lam = side == 0 ? lamL : lamR;
            const double w = side == 0 ? wL : 1.0 - wL;
            const double dni = 1.0 / qs[RH];
            const double vel[3] = {qs[MX] * dni, qs[MY] * dni, qs[MZ] * dni};
#pragma unroll
            for (int v = PXX; v < NQ; ++v) lam[v] = 0.0;
            if (src.cell < 0) continue;
#pragma unroll
            for (int i = 0; i < 3; ++i)
                if ((src.mask >> PN[i]) & 1u) lam[PN[i]] = w * fma(lamF[EN], vel[i], lamF[MX + i]);
        }

    }
    // a ghost made from a cell's own trace hands its adjoint to that trace
    if (ghostL_from_R) {
#pragma unroll
        for (int v = 0; v < NQ; ++v) { lamR[v] += lamL[v]; lamL[v] = 0.0; }
    }
    if (ghostR_from_L) {
#pragma unroll
        for (int v = 0; v < NQ; ++v) { lamL[v] += lamR[v]; lamR[v] = 0.0; }
    }
    const long long nfd = (long long)ex * ey * (DIR == 2 ? B.nfp[2] : n2);
    double* tb = tadj + 2 * B.fbase[DIR];
#pragma unroll
    for (int v = 0; v < NQ; ++v) {
        tb[((long long)(0 * NQ + v) * TB::NF + P) * nfd + lf] = lamL[v];
        tb[((long long)(1 * NQ + v) * TB::NF + P) * nfd + lf] = lamR[v];
    }
}

template <class TB, int DIR, int MODE>
__global__ void __launch_bounds__(ADJ_TPB) k_face_adj(const double* __restrict__ Q, const double* __restrict__ mu,
                                                      double* __restrict__ tadj, AdjArgs a) {
    const long long gf = (long long)blockIdx.x * ADJ_TPB + threadIdx.x;
    if (gf >= a.G.nface[DIR]) return;
    const int p = blockIdx.y;
    sfor<TB::NF>([&](auto pp) {
        constexpr int P = decltype(pp)::value;
        if (p == P) face_adj_point<TB, DIR, P, MODE>(Q, mu, tadj, a, gf);
    });
}

// one cell of the cell pass; returns mu . dR/dcoll of the cell when
// a.cpart is set (ivis 0: the relaxation -coll P; ivis 2: the source
// coll rho (v v - |v|^2/3); R of ivis 1 does not depend on coll)
template <class TB, int MODE>
__device__ __forceinline__ double cell_adj_body(const double* __restrict__ Q, const double* __restrict__ mu,
                                                const double* __restrict__ tadj, double* __restrict__ out,
                                                const AdjArgs& a, long long le) {
    constexpr int NB = TB::NB, NF = TB::NF, NPG = TB::NPG;
    const Phys& ph = a.ph;
    double cr = 0.0;
    const Box& B = a.G.boxes[0];
    const long long nc = B.ncell;
    double nu[NB][NQ];
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int v = 0; v < NQ; ++v) nu[b][v] = 0.0;
    // ---- traces: transpose of the trace evaluation of both faces per direction
    const int n0 = B.n[0], n1 = B.n[1];
    const int c[3] = {(int)(le % n0), (int)((le / n0) % n1), (int)(le / ((long long)n0 * n1))};
    sfor<3>([&](auto dd) {
        constexpr int d = decltype(dd)::value;
        const int e0 = d == 0 ? B.nfp[0] : B.n[0], e1 = d == 1 ? B.nfp[1] : B.n[1], e2 = d == 2 ? B.nfp[2] : B.n[2];
        const long long nfd = (long long)e0 * e1 * e2;
        int hi = c[d] + 1;
        if (B.nfp[d] == B.n[d] && hi == B.n[d]) hi = 0;
        const int lo = c[d];
        int a0 = d == 0 ? lo : c[0], a1 = d == 1 ? lo : c[1], a2 = d == 2 ? lo : c[2];
        const long long fm = (long long)a0 + (long long)e0 * (a1 + (long long)e1 * a2);
        a0 = d == 0 ? hi : c[0]; a1 = d == 1 ? hi : c[1]; a2 = d == 2 ? hi : c[2];
        const long long fp = (long long)a0 + (long long)e0 * (a1 + (long long)e1 * a2);
        const double* tb = tadj + 2 * B.fbase[d];
        sfor<NF>([&](auto pp) {
            constexpr int p = decltype(pp)::value;
#pragma unroll
            for (int v = 0; v < NQ; ++v) {
                const double lm = tb[((long long)(1 * NQ + v) * NF + p) * nfd + fm];   // minus face: R slot
                const double lp = tb[((long long)(0 * NQ + v) * NF + p) * nfd + fp];   // plus face: L slot
                sfor<NB>([&](auto bb) {
                    constexpr int b = decltype(bb)::value;
                    constexpr double cm = ftab<TB, d, 0>(p, b);
                    constexpr double cp = ftab<TB, d, 1>(p, b);
                    if constexpr (cm != 0.0) nu[b][v] = fma(cm, lm, nu[b][v]);
                    if constexpr (cp != 0.0) nu[b][v] = fma(cp, lp, nu[b][v]);
                });
            }
        });
    });
    // ---- volume quadrature and sources: R -= sum_g VD di F_d(u(g)) + SRC s(u(g))
    const double di[3] = {B.di[0], B.di[1], B.di[2]};
    const bool src_lin = ph.ivis == 0, src_bf = ph.body_force != 0.0;
    const Dual S0[6] = {Dual(0.0), Dual(0.0), Dual(0.0), Dual(0.0), Dual(0.0), Dual(0.0)};
    sfor_seq<NPG>([&](auto gg) {
        constexpr int g = decltype(gg)::value;
        double u[NQ];
        sfor<NQ>([&](auto vv) {
            constexpr int v = decltype(vv)::value;
            double s = 0.0;
            sfor<NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                constexpr double cI = TB::INT(g, b);
                if constexpr (cI != 0.0) s = fma(cI, Q[(long long)(b * NQ + v) * nc + le], s);
            });
            u[v] = s;
        });
        // adjoints of the point fluxes and point sources at g
        double lamF[3][NQ], lamS[NQ];
#pragma unroll
        for (int v = 0; v < NQ; ++v) {
            double a0 = 0.0, a1 = 0.0, a2 = 0.0, as = 0.0;
            sfor<NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                const double m = mu[(long long)(b * NQ + v) * nc + le];
                constexpr double c0 = TB::VX(g, b), c1 = TB::VY(g, b), c2 = TB::VZ(g, b), cs = TB::SRC(g, b);
                if constexpr (c0 != 0.0) a0 = fma(c0, m, a0);
                if constexpr (c1 != 0.0) a1 = fma(c1, m, a1);
                if constexpr (c2 != 0.0) a2 = fma(c2, m, a2);
                if constexpr (cs != 0.0) as = fma(cs, m, as);
            });
            lamF[0][v] = -di[0] * a0;
            lamF[1][v] = -di[1] * a1;
            lamF[2][v] = -di[2] * a2;
            lamS[v] = -as;
        }
        if (a.cpart) {   // mu . dR/dcoll at g: sum_v lamS[v] ds_v/dcoll
            if (ph.ivis == 0) {
#pragma unroll
                for (int v = PXX; v < NQ; ++v) cr = fma(lamS[v], -u[v], cr);
            } else if (ph.ivis == 2) {
                Phys p1 = ph;
                p1.coll = 1.0;
                double sv[6];
                ten_moment_source<double>(p1, primitives(ph, u), sv);
#pragma unroll
                for (int m = 0; m < 6; ++m) cr = fma(lamS[PXX + m], sv[m], cr);
            }
        }
        double lamu[NQ];
        if constexpr (MODE == ADJ_GEN) {
            // one dual pass per column: the point fluxes of the three
            // directions (with the stochastic stress of the forward cell
            // kernel's draw, kind 3 + d, site le, point g) and the sources
            double Sn[3][6];
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int c = 0; c < 6; ++c) Sn[d][c] = 0.0;
            if (ph.llns) {
                const NoiseCtr nc{*a.nstep, a.nstage};
#pragma unroll
                for (int d = 0; d < 3; ++d) random_stress<double>(ph, B.seed, nc, 3 + d, (unsigned long long)le, g, Sn[d]);
            }
#pragma unroll 1
            for (int jv = 0; jv < NQ; ++jv) {
                Dual ud[NQ];
#pragma unroll
                for (int v = 0; v < NQ; ++v) ud[v] = Dual(u[v], v == jv ? 1.0 : 0.0);
                const Prim<Dual> w = primitives(ph, ud);
                double acc = 0.0;
                sfor<3>([&](auto dd) {
                    constexpr int d = decltype(dd)::value;
                    const Dual Sd[6] = {Dual(Sn[d][0]), Dual(Sn[d][1]), Dual(Sn[d][2]),
                                        Dual(Sn[d][3]), Dual(Sn[d][4]), Dual(Sn[d][5])};
                    Dual f[NQ];
                    point_flux<Dual, d>(ph, ud, w, Sd, f);
#pragma unroll
                    for (int v = 0; v < NQ; ++v) acc = fma(lamF[d][v], f[v].d, acc);
                });
                if (ph.ivis == 2) {   // sources.f90:51-69
                    Dual sv[6];
                    ten_moment_source<Dual>(ph, w, sv);
#pragma unroll
                    for (int m = 0; m < 6; ++m) acc = fma(lamS[PXX + m], sv[m].d, acc);
                }
                if (src_lin && jv >= PXX) acc = fma(lamS[jv], -ph.coll, acc);   // sources.f90:37-43
                if (src_bf) {    // body force (no reference counterpart): linear in rho and m_x
                    if (jv == RH) acc = fma(lamS[MX], ph.body_force, acc);
                    if (jv == MX) acc = fma(lamS[EN], ph.body_force, acc);
                }
                lamu[jv] = acc;
            }
        } else if constexpr (MODE == ADJ_REV) {
            // one reverse sweep of the primitives and the three point fluxes
            // (dg_flux_vjp.cuh), then the linear sources
#pragma unroll
            for (int v = 0; v < NQ; ++v) lamu[v] = 0.0;
            const SideRev sp = side_primal(ph, u);
            sfor<3>([&](auto dd) {
                constexpr int d = decltype(dd)::value;
                point_flux_rev<d>(ph, u, sp, lamF[d], lamu);
            });
            if (src_lin) {   // sources.f90:37-43
#pragma unroll
                for (int v = PXX; v < NQ; ++v) lamu[v] = fma(lamS[v], -ph.coll, lamu[v]);
            }
            if (src_bf) {    // body force (no reference counterpart): linear in rho and m_x
                lamu[RH] = fma(lamS[MX], ph.body_force, lamu[RH]);
                lamu[MX] = fma(lamS[EN], ph.body_force, lamu[MX]);
            }
        } else {
        // hydro columns (rh..en): one dual pass each; stress columns in closed
        // form (the stresses enter the point fluxes linearly: f_d[M_i] +=
        // P_{d i}, f_d[E] += P_{d i} v_i, and the ivis-0 source -coll P)
#pragma unroll 1
        for (int jv = 0; jv <= EN; ++jv) {
            Dual ud[NQ];
#pragma unroll
            for (int v = 0; v < NQ; ++v) ud[v] = Dual(u[v], v == jv ? 1.0 : 0.0);
            const Prim<Dual> w = primitives(ph, ud);
            double acc = 0.0;
            sfor<3>([&](auto dd) {
                constexpr int d = decltype(dd)::value;
                Dual f[NQ];
                point_flux<Dual, d>(ph, ud, w, S0, f);
#pragma unroll
                for (int v = 0; v < NQ; ++v) acc = fma(lamF[d][v], f[v].d, acc);
            });
            // body force (no reference counterpart): linear in rho and m_x
            if (src_bf) {
                if (jv == RH) acc = fma(lamS[MX], ph.body_force, acc);
                if (jv == MX) acc = fma(lamS[EN], ph.body_force, acc);
            }
            lamu[jv] = acc;
        }
        {
            const double dni = 1.0 / u[RH];
            const double vel[3] = {u[MX] * dni, u[MY] * dni, u[MZ] * dni};
            constexpr int PD[3][3] = {{PXX, PXY, PXZ}, {PXY, PYY, PYZ}, {PXZ, PYZ, PZZ}};
#pragma unroll
            for (int v = PXX; v < NQ; ++v) lamu[v] = src_lin ? lamS[v] * -ph.coll : 0.0;   // sources.f90:37-43
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int i = 0; i < 3; ++i) lamu[PD[d][i]] += fma(lamF[d][EN], vel[i], lamF[d][MX + i]);
        }
        }
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            constexpr double cI = TB::INT(g, b);
            if constexpr (cI != 0.0) {
#pragma unroll
                for (int v = 0; v < NQ; ++v) nu[b][v] = fma(cI, lamu[v], nu[b][v]);
            }
        });
    });
    const double dt = a.st[0].dt;
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int v = 0; v < NQ; ++v) {
            const long long ix = (long long)(b * NQ + v) * nc + le;
            out[ix] = a.mode == 0 ? nu[b][v] : mu[ix] - dt * nu[b][v];
        }
    return cr;
}

template <class TB, int MODE>
__global__ void __launch_bounds__(ADJ_TPB) k_cell_adj(const double* __restrict__ Q, const double* __restrict__ mu,
                                                      const double* __restrict__ tadj, double* __restrict__ out, AdjArgs a) {
    const long long le = (long long)blockIdx.x * ADJ_TPB + threadIdx.x;
    double cr = 0.0;
    if (le < a.G.ncell) cr = cell_adj_body<TB, MODE>(Q, mu, tadj, out, a, le);
    if (a.cpart) {   // block partial of mu . dR/dcoll, summed in a fixed order
        __shared__ double ws[ADJ_TPB / 32];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cr += __shfl_down_sync(0xffffffffu, cr, o);
        if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = cr;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
#pragma unroll
            for (int w = 0; w < ADJ_TPB / 32; ++w) t += ws[w];
            a.cpart[blockIdx.x] = t;
        }
    }
}

// the cell pass of one basis; the reverse-sweep and the dual-number (check
// path) variants are compiled in units of their own (adj_f64_nb*_cell.cu,
// adj_f64_nb*_dual.cu), the cell kernels being the slowest to compile
template <int NB, int NQD, int MODE>
cudaError_t cell_adj_launch(const double* Q, const double* mu, const double* tadj, double* out, const AdjArgs& a,
                            cudaStream_t s) {
    using TB = hermes_tab::Tab<NB, NQD>;
    if (a.G.ncell > 0) {
        const unsigned nblk = (unsigned)((a.G.ncell + ADJ_TPB - 1) / ADJ_TPB);
        k_cell_adj<TB, MODE><<<nblk, ADJ_TPB, 0, s>>>(Q, mu, tadj, out, a);
    }
    return cudaGetLastError();
}
cudaError_t cell_adj_dual(int nb, const double* Q, const double* mu, const double* tadj, double* out,
                          const AdjArgs& a, cudaStream_t s);
cudaError_t cell_adj_rev(int nb, const double* Q, const double* mu, const double* tadj, double* out,
                         const AdjArgs& a, cudaStream_t s);
cudaError_t cell_adj_gen(int nb, const double* Q, const double* mu, const double* tadj, double* out,
                         const AdjArgs& a, cudaStream_t s);

// k_limit_adj: lam_in = (dL/dq)^T lam_out for the positivity limiter L of
// flux.f90:1077-1164 (limit_cell, the forward kernels' own code), one thread
// per cell.  The limiter is cell-local and touches only the hydro rows; where
// the forward bound test shows it inactive the map is the identity, elsewhere
// one dual-number pass per hydro coefficient (5 nb columns) runs limit_cell
// and gives the derivative of its active branch (the arg-min face point, the
// clamp of theta, the floors).  lam_out is read in full before lam_in is
// written, so the two may be one buffer.
template <class TB>
__global__ void __launch_bounds__(ADJ_TPB) k_limit_adj(const double* __restrict__ Q, const double* lam_out,
                                                       double* lam_in, Geom G, Phys ph) {
    constexpr int NB = TB::NB;
    const long long le = (long long)blockIdx.x * ADJ_TPB + threadIdx.x;
    if (le >= G.ncell) return;
    const long long nc = G.boxes[0].ncell;
    double q[5][NB], lo[5][NB];
    sfor<5>([&](auto vv) {
        constexpr int v = decltype(vv)::value;
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            q[v][b] = Q[(long long)(b * NQ + v) * nc + le];
            lo[v][b] = lam_out[(long long)(b * NQ + v) * nc + le];
        });
    });
    if (lam_in != lam_out) {   // stress rows: the identity
        for (int b = 0; b < NB; ++b)
#pragma unroll
            for (int v = PXX; v < NQ; ++v) lam_in[(long long)(b * NQ + v) * nc + le] = lam_out[(long long)(b * NQ + v) * nc + le];
    }
    if (q[RH][0] >= ph.rh_floor && limit_bound_clear<TB, double>(ph, q)) {
        if (lam_in != lam_out)
            sfor<5>([&](auto vv) {
                constexpr int v = decltype(vv)::value;
                sfor<NB>([&](auto bb) {
                    constexpr int b = decltype(bb)::value;
                    lam_in[(long long)(b * NQ + v) * nc + le] = lo[v][b];
                });
            });
        return;
    }
#pragma unroll 1
    for (int col = 0; col < 5 * NB; ++col) {
        const int cv = col / NB, cb = col % NB;
        Dual qd[5][NB];
        sfor<5>([&](auto vv) {
            constexpr int v = decltype(vv)::value;
            sfor<NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                qd[v][b] = Dual(q[v][b], (v == cv && b == cb) ? 1.0 : 0.0);
            });
        });
        limit_cell<TB, Dual>(ph, qd);
        double acc = 0.0;
        sfor<5>([&](auto vv) {
            constexpr int v = decltype(vv)::value;
            sfor<NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                acc = fma(lo[v][b], qd[v][b].d, acc);
            });
        });
        lam_in[(long long)(cb * NQ + cv) * nc + le] = acc;
    }
}

template <int NB, int NQD>
cudaError_t limit_adj_launch(const double* Q, const double* lam_out, double* lam_in, const Geom& G, const Phys& ph,
                             cudaStream_t s) {
    using TB = hermes_tab::Tab<NB, NQD>;
    if (G.ncell > 0) {
        const unsigned nblk = (unsigned)((G.ncell + ADJ_TPB - 1) / ADJ_TPB);
        k_limit_adj<TB><<<nblk, ADJ_TPB, 0, s>>>(Q, lam_out, lam_in, G, ph);
    }
    return cudaGetLastError();
}

// launcher of one basis: the three face-adjoint passes, then the cell pass
template <int NB, int NQD>
cudaError_t adj_launch(const double* Q, const double* mu, double* tadj, double* out, const AdjArgs& a, cudaStream_t s) {
    using TB = hermes_tab::Tab<NB, NQD>;
    for (int d = 0; d < 3; ++d) {
        const long long n = a.G.nface[d];
        if (n <= 0) continue;
        dim3 grid((unsigned)((n + ADJ_TPB - 1) / ADJ_TPB), TB::NF);
        if (a.dual == ADJ_GEN) {   // one dual pass per column (ivis 2, Tait EOS)
            if (d == 0) k_face_adj<TB, 0, ADJ_GEN><<<grid, ADJ_TPB, 0, s>>>(Q, mu, tadj, a);
            else if (d == 1) k_face_adj<TB, 1, ADJ_GEN><<<grid, ADJ_TPB, 0, s>>>(Q, mu, tadj, a);
            else k_face_adj<TB, 2, ADJ_GEN><<<grid, ADJ_TPB, 0, s>>>(Q, mu, tadj, a);
        } else if (a.dual) {   // forward-mode dual passes (the check on the reverse sweep)
            if (d == 0) k_face_adj<TB, 0, ADJ_DUAL><<<grid, ADJ_TPB, 0, s>>>(Q, mu, tadj, a);
            else if (d == 1) k_face_adj<TB, 1, ADJ_DUAL><<<grid, ADJ_TPB, 0, s>>>(Q, mu, tadj, a);
            else k_face_adj<TB, 2, ADJ_DUAL><<<grid, ADJ_TPB, 0, s>>>(Q, mu, tadj, a);
        } else {
            if (d == 0) k_face_adj<TB, 0, ADJ_REV><<<grid, ADJ_TPB, 0, s>>>(Q, mu, tadj, a);
            else if (d == 1) k_face_adj<TB, 1, ADJ_REV><<<grid, ADJ_TPB, 0, s>>>(Q, mu, tadj, a);
            else k_face_adj<TB, 2, ADJ_REV><<<grid, ADJ_TPB, 0, s>>>(Q, mu, tadj, a);
        }
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (a.dual == ADJ_GEN) return cell_adj_gen(NB, Q, mu, tadj, out, a, s);
    if (a.dual) return cell_adj_dual(NB, Q, mu, tadj, out, a, s);
    return cell_adj_rev(NB, Q, mu, tadj, out, a, s);
}

}  // namespace hermes

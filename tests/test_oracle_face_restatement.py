"""A second, independent restatement of the reference's face flux and
sources, in numpy, read afresh from the Fortran, against the C oracle.

For a piecewise-constant state (cell averages only) on a periodic line of
three cells, every face point of a face carries the same left and right
states and the transverse faces see the same cell on both sides, so the
cell-average row of glflux - source (flux.f90:963-965, sources.f90:36-69) is

    dxi (F(q_i, q_i+1) - F(q_i-1, q_i)) - S(q_i)

with F the numerical flux of one face point.  That isolates, per direction:
  * the point flux flux_calc_pnts_r (flux.f90:23-190) for ivis 0/1 (the
    stress fluxes colvis-scaled velocities) and ivis 2 (the 10-moment terms),
    with P and P_10 floored there but not in HLLC;
  * HLLC (flux.f90:466-647): the wave-speed estimates, the stale 1/rho of the
    last point of the call in the Tait sound speeds (ieos 2), the zero
    denominators set to rh_floor, Batten's star states, and the four branch
    tests applied one after another, so a later one overrides an earlier one
    (the tie S_M = 0 takes F_R*);
  * the Roe variant of the monolithic 10-moment code
    (src/ces/10_moment/dg_3D_hydro_lqc_SEAN.f90:1614-1789) with its
    half-weighted pressure term in the Roe enthalpy;
  * the central flux on every variable HLLC does not set, with the freezing
    speed max(cfcal(L), cfcal(R)) as dissipation for ivis 2 only (cfrx is set
    nowhere else, flux.f90:248-258; cfcal flux.f90:1029-1072);
  * the sources of ivis 0 (-coll P_ij) and ivis 2 (coll rho (v_i v_j -
    delta_ij |v|^2/3)).
The two restatements are written separately (the C one per face with the
kernels' layout, this one per state from the Fortran's formulas), so their
agreement to rounding checks the transcription of each against the other."""
import math

import numpy as np
import pytest

from hermeshd_gb300 import config

RH, MX, MY, MZ, EN, PXX, PYY, PZZ, PXY, PXZ, PYZ = range(11)
# stress index of the pair (i, j) of directions
PIJ = {(0, 0): PXX, (1, 1): PYY, (2, 2): PZZ, (0, 1): PXY, (1, 0): PXY, (0, 2): PXZ, (2, 0): PXZ,
       (1, 2): PYZ, (2, 1): PYZ}


def philox4x32_10(ctr, key):
    """Philox-4x32-10 (Salmon et al., SC'11) on Python integers."""
    c0, c1, c2, c3 = ctr
    k0, k1 = key
    M = 0xFFFFFFFF
    for _ in range(10):
        p0 = 0xD2511F53 * c0
        p1 = 0xCD9E8D57 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & M, p1 & M, ((p0 >> 32) ^ c3 ^ k1) & M, p0 & M
        k0 = (k0 + 0x9E3779B9) & M
        k1 = (k1 + 0xBB67AE85) & M
    return c0, c1, c2, c3


def stress_sample(cfg, step, stage, kind, site, pt):
    """The stochastic stress (Sxx, Syy, Szz, Sxy, Sxz, Syz) of one point of
    one flux call, restated from the documented counter scheme: key = seed,
    counter = (site, pt | kind << 8 | block << 12 | stage << 16, step low,
    step high); each 32-bit word a uniform (w + 1/2) 2^-32; three Box-Muller
    pairs of the first six words give the diagonal and off-diagonal normals;
    S = eta (G_ii - tr G / 3) + zeta tr G on the diagonal, eta G_ij off it
    (random.f90:124-141 with its nine normals' six independent combinations
    drawn directly)."""
    key = (cfg.seed & 0xFFFFFFFF, cfg.seed >> 32)
    w = []
    for blk in range(2):
        ctr = (site & 0xFFFFFFFF, (pt & 0xFF) | ((kind & 0xF) << 8) | ((blk & 0xF) << 12) | ((stage & 0xFFFF) << 16),
               step & 0xFFFFFFFF, step >> 32)
        w += philox4x32_10(ctr, key)
    G = []
    for k in range(3):
        u1, u2 = (w[2 * k] + 0.5) * 2.0 ** -32, (w[2 * k + 1] + 0.5) * 2.0 ** -32
        r = math.sqrt(-2.0 * math.log(u1))
        G += [r * math.cos(2 * math.pi * u2), r * math.sin(2 * math.pi * u2)]
    tr = G[0] + G[1] + G[2]
    e, z = cfg.eta_sd, cfg.zeta_sd
    return np.array([e * (G[0] - tr / 3) + z * tr, e * (G[1] - tr / 3) + z * tr, e * (G[2] - tr / 3) + z * tr,
                     e * G[3], e * G[4], e * G[5]])


def point_flux(cfg, q, d, S=None):
    """flux_calc_pnts_r (flux.f90:23-190) of one state in direction d (0, 1, 2),
    with the stochastic stress S (Sxx, Syy, Szz, Sxy, Sxz, Syz) or none."""
    g = cfg.aindex
    dn, M, Ener = q[RH], q[MX:MZ + 1], q[EN]
    P_ = {k: q[v] for k, v in PIJ.items()}
    dni = 1.0 / dn
    v = M * dni
    smsq = M[0] ** 2 + M[1] ** 2 + M[2] ** 2
    P = (g - 1) * (Ener - 0.5 * dni * smsq)
    P10 = (1.0 / 3.0) * (q[PXX] + q[PYY] + q[PZZ] - dni * smsq)
    if cfg.ieos == 2:
        P = cfg.P_1 * (dn ** 7.2 - 1.0) + cfg.P_base + P
    Pfl = cfg.T_floor * cfg.rh_floor
    P = max(P, Pfl)
    P10 = max(P10, Pfl)
    f = np.zeros(11)
    f[RH] = M[d]
    others = [j for j in range(3) if j != d]
    S_ = {k: (0.0 if S is None else S[v - PXX]) for k, v in PIJ.items()}
    for j in range(3):
        if cfg.ivis in (0, 1):
            f[MX + j] = M[j] * v[d] + (P if j == d else 0.0) + P_[(j, d)] - S_[(j, d)]
        else:
            f[MX + j] = (P_[(d, d)] - P10 + P) if j == d else P_[(j, d)]
    if cfg.ivis == 3:      # Grad closure: the energy tensor E_ij does no work (ten_moment.f90:969)
        f[EN] = (Ener + P) * v[d]
    else:
        f[EN] = (Ener + P) * v[d] + (P_[(d, d)] - S_[(d, d)]) * v[d] + \
            (P_[(d, others[0])] - S_[(d, others[0])]) * v[others[0]] + \
            (P_[(d, others[1])] - S_[(d, others[1])]) * v[others[1]]
    cv = cfg.colvis
    if cfg.ivis in (0, 1):
        for j in range(3):
            f[PIJ[(j, j)]] = (4.0 / 3.0) * cv * v[d] if j == d else -(2.0 / 3.0) * cv * v[d]
        for (a, b) in ((0, 1), (0, 2), (1, 2)):
            f[PIJ[(a, b)]] = cv * v[b if a == d else a] if d in (a, b) else 0.0
    else:                  # ivis 2, and ivis 3 with E_ij (ten_moment.f90:895-1000)
        vx, vy, vz = v
        Mx, My, Mz = M
        Pxx, Pyy, Pzz, Pxy, Pxz, Pyz = (q[k] for k in (PXX, PYY, PZZ, PXY, PXZ, PYZ))
        if d == 0:
            f[PXX] = vx * (3 * Pxx - 2 * vx * Mx)
            f[PYY] = 2 * vy * (Pxy - vy * Mx) + vx * Pyy
            f[PZZ] = 2 * vz * (Pxz - vz * Mx) + vx * Pzz
            f[PXY] = 2 * vx * (Pxy - vy * Mx) + vy * Pxx
            f[PXZ] = 2 * vx * (Pxz - vz * Mx) + vz * Pxx
            f[PYZ] = vx * Pyz + vy * Pxz + vz * Pxy - 2 * vy * vz * Mx
        elif d == 1:
            f[PXX] = 2 * vx * (Pxy - vx * My) + vy * Pxx
            f[PYY] = vy * (3 * Pyy - 2 * vy * My)
            f[PZZ] = 2 * vz * (Pyz - vz * My) + vy * Pzz
            f[PXY] = 2 * vy * (Pxy - vx * My) + vx * Pyy
            f[PXZ] = vx * Pyz + vy * Pxz + vz * Pxy - 2 * vx * vz * My
            f[PYZ] = 2 * vy * (Pyz - vz * My) + vz * Pyy
        else:
            f[PXX] = 2 * vx * (Pxz - vx * Mz) + vz * Pxx
            f[PYY] = 2 * vy * (Pyz - vy * Mz) + vz * Pyy
            f[PZZ] = vz * (3 * Pzz - 2 * vz * Mz)
            f[PXY] = vx * Pyz + vy * Pxz + vz * Pxy - 2 * vx * vy * Mz
            f[PXZ] = 2 * vz * (Pxz - vx * Mz) + vx * Pzz
            f[PYZ] = 2 * vz * (Pyz - vy * Mz) + vy * Pzz
    return f


def cfcal(cfg, q, d):
    """Freezing speed |v_d| + c_s (flux.f90:1029-1072; for ivis 3
    ten_moment.f90:1721-1754, the same with the pressure of E_ij)."""
    dn = q[RH]
    dni = 1.0 / dn
    v = q[MX:MZ + 1] * dni
    if cfg.ivis >= 2:
        P = (1.0 / 3.0) * (q[PXX] + q[PYY] + q[PZZ] - dn * (v[0] ** 2 + v[1] ** 2 + v[2] ** 2))
    else:
        P = (cfg.aindex - 1) * (q[EN] - 0.5 * dn * (v[0] ** 2 + v[1] ** 2 + v[2] ** 2))
    cs = math.sqrt(cfg.aindex * P * dni) if cfg.ieos == 1 else math.sqrt(7.2 * cfg.P_1 * dn ** 6.2)
    return abs(v[d]) + cs


def hllc(cfg, qL, qR, fL, fR, d, stale=True, rho_last=None):
    """flux_hllc (flux.f90:466-647) of one face point.  The Tait sound speeds
    take the stale 1/rho of the last point of the reference's call, the right
    state at the face's last point: rho_last, or this point's right state when
    every point of the face carries the same states.  Returns the fluxes of
    rh, mx, my, mz, en."""
    g, ieos = cfg.aindex, cfg.ieos
    ipar, ip1, ip2 = [(MX, MY, MZ), (MY, MZ, MX), (MZ, MX, MY)][d]
    ivar = (RH, ipar, ip1, ip2, EN)
    side = []
    for q in (qL, qR):
        rho = q[RH]
        ri = 1.0 / rho
        vv = (q[ipar] * ri, q[ip1] * ri, q[ip2] * ri)
        qsq = vv[0] ** 2 + vv[1] ** 2 + vv[2] ** 2
        p = (g - 1) * (q[EN] - 0.5 * rho * qsq)
        if ieos == 2:
            p = cfg.P_1 * (rho ** 7.2 - 1.0) + cfg.P_base + p
        side.append((rho, vv, p))
    (rL, vL, pL), (rR, vR, pR) = side
    rho_i = 1.0 / (rR if rho_last is None else rho_last)   # the last point of the call: a right state

    def speed(rho, p):
        if ieos == 2:
            return math.sqrt(7.2 * cfg.P_1 * rho ** 6.2 + p * (rho_i if stale else 1.0 / rho))
        return math.sqrt(g * p / rho)
    csL = vL[0] - speed(rL, pL)               # lambda_M(Q_l)
    csR = vR[0] + speed(rR, pR)               # lambda_P(Q_r)
    qsL = vR[0] - speed(rR, pR)               # lambda_M(Q_r)
    qsR = vL[0] + speed(rL, pL)               # lambda_P(Q_l)
    SL, SR = min(csL, qsL), max(csR, qsR)
    num = rR * vR[0] * (SR - vR[0]) - rL * vL[0] * (SL - vL[0])
    num = num + pL - pR
    den = rR * (SR - vR[0]) - rL * (SL - vL[0])
    if den == 0.0:
        den = cfg.rh_floor
    SM = num / den
    pstar = rL * (vL[0] - SL) * (vL[0] - SM) + pL

    def fstar(q, rho, vv, p, f, S):
        dd = S - SM
        if dd == 0.0:
            dd = cfg.rh_floor
        si = 1.0 / dd
        sq = S - vv[0]
        Qs = (rho * sq * si,
              (sq * q[ipar] + pstar - p) * si,
              sq * q[ip1] * si,
              sq * q[ip2] * si,
              (sq * q[EN] - p * vv[0] + pstar * SM) * si)
        return [f[ivar[m]] + S * (Qs[m] - q[ivar[m]]) for m in range(5)]
    FLs = fstar(qL, rL, vL, pL, fL, SL)
    FRs = fstar(qR, rR, vR, pR, fR, SR)
    out = [None] * 5
    if SL > 0.0:
        out = [fL[ivar[m]] for m in range(5)]
    if SL <= 0.0 and 0.0 < SM:
        out = FLs
    if SM <= 0.0 and 0.0 <= SR:
        out = FRs
    if SR < 0.0:
        out = [fR[ivar[m]] for m in range(5)]
    res = np.zeros(5)
    for m in range(5):
        res[ivar[m]] = out[m]                  # fhllc(i4, ivar(ieq)): natural variable order
    return res, (SL, SM, SR)


def roe(cfg, qL, qR, fL, fR, d):
    """flux_roe of the monolithic 10-moment code
    (src/ces/10_moment/dg_3D_hydro_lqc_SEAN.f90:1614-1789): the central flux
    minus half the Roe-matrix flux increment, with that code's direction
    triples mxa/mya/mza (:236-244), cp = gamma/(gamma-1) (:81) and its
    Roe-averaged enthalpy 0.5 sqrt(rho) (v^2 + cp P/rho) (:1676).  None where
    the Roe sound speed squared is not positive."""
    g = cfg.aindex
    am1 = g - 1.0
    cp = g / (g - 1.0)
    mxa, mya, mza = [(MX, MY, MZ), (MY, MZ, MX), (MZ, MX, MY)][d]
    skr, swr = [], []
    for q in (qL, qR):
        dnii = 1.0 / q[RH]
        vels = (q[mxa] * dnii, q[mya] * dnii, q[mza] * dnii)
        vsq = vels[0] ** 2 + vels[1] ** 2 + vels[2] ** 2
        Pri = am1 * (q[EN] - 0.5 * q[RH] * vsq)
        sk = math.sqrt(q[RH])
        skr.append(sk)
        swr.append((sk * vels[0], sk * vels[1], sk * vels[2], 0.5 * sk * (vsq + cp * Pri / q[RH])))
    Qri = 1.0 / qL[RH]
    delrho = qR[RH] * Qri - 1.0
    dele = (qR[EN] - qL[EN]) * Qri
    dm1 = (qR[mxa] - qL[mxa]) * Qri
    dm2 = (qR[mya] - qL[mya]) * Qri
    dm3 = (qR[mza] - qL[mza]) * Qri
    dwr = [0.5 * (swr[1][j] + swr[0][j]) for j in range(4)]
    dsk = 0.5 * (skr[1] + skr[0])
    vc = (dwr[0] / dsk, dwr[1] / dsk, dwr[2] / dsk)
    hc = dwr[3] / dsk
    vcsq = vc[0] * vc[0] + vc[1] * vc[1] + vc[2] * vc[2]
    asq = am1 * (hc - 0.5 * vcsq)
    if asq <= 0.0:
        return None
    sc = math.sqrt(asq)
    lam = (abs(vc[0] - sc), abs(vc[0] + sc), abs(vc[0]), abs(vc[0]), abs(vc[0]))
    # eigenvectors as columns, rows ordered (rho, E, m_par, m_perp1, m_perp2)
    evec = np.zeros((5, 5))
    evec[0, 0] = evec[0, 1] = evec[0, 2] = 1.0
    evec[3, 3] = evec[4, 4] = 1.0
    evec[1, 0], evec[2, 0], evec[3, 0], evec[4, 0] = hc - sc * vc[0], vc[0] - sc, vc[1], vc[2]
    evec[1, 1], evec[2, 1], evec[3, 1], evec[4, 1] = hc + sc * vc[0], vc[0] + sc, vc[1], vc[2]
    evec[1, 2], evec[2, 2], evec[3, 2], evec[4, 2] = 0.5 * vcsq, vc[0], vc[1], vc[2]
    evec[1, 3], evec[1, 4] = vc[1], vc[2]
    ea2i = am1 / asq
    vcdel = vc[0] * dm1 + vc[1] * dm2 + vc[2] * dm3 - dele
    a9e = 0.5 * ea2i * (0.5 * vcsq * delrho - vcdel)
    sk9 = 0.5 * (dm1 - vc[0] * delrho) / sc
    a9 = (a9e - sk9, a9e + sk9, ea2i * ((hc - vcsq) * delrho + vcdel), dm2 - vc[1] * delrho, dm3 - vc[2] * delrho)
    df = np.zeros(5)
    for j in range(5):                         # the reference's accumulation order
        for r in range(5):
            df[r] = df[r] + a9[j] * lam[j] * evec[r, j]
    df = df * qL[RH]
    res = np.zeros(5)
    res[RH] = 0.5 * (fL[RH] + fR[RH] - df[0])
    res[EN] = 0.5 * (fL[EN] + fR[EN] - df[1])
    res[mxa] = 0.5 * (fL[mxa] + fR[mxa] - df[2])
    res[mya] = 0.5 * (fL[mya] + fR[mya] - df[3])
    res[mza] = 0.5 * (fL[mza] + fR[mza] - df[4])
    return res


def face_flux(cfg, qL, qR, d, stale=True, rho_last=None, SL=None, SR=None):
    fL, fR = point_flux(cfg, qL, d, SL), point_flux(cfg, qR, d, SR)
    cfr = max(cfcal(cfg, qL, d), cfcal(cfg, qR, d)) if cfg.ivis >= 2 else 0.0
    F = 0.5 * (fL + fR) - 0.5 * cfr * (qR - qL)
    waves = None
    if cfg.ihllc == 1:
        F[RH:EN + 1], waves = hllc(cfg, qL, qR, fL, fR, d, stale, rho_last)
    elif cfg.ihllc == 2:
        r = roe(cfg, qL, qR, fL, fR, d)
        assert r is not None                   # the cases here keep the Roe sound speed real
        F[RH:EN + 1] = r
    return F, waves


def source(cfg, q):
    """sources.f90:36-69 at one point, plus the x body force (a term of this
    implementation, no reference counterpart: rho g on m_x, m_x g on E)."""
    s = np.zeros(11)
    if cfg.body_force != 0.0:
        s[MX] = q[RH] * cfg.body_force
        s[EN] = q[MX] * cfg.body_force
    if cfg.ivis == 0:
        s[PXX:] = -cfg.coll * q[PXX:]
    elif cfg.ivis == 2:
        dn = q[RH]
        v = q[MX:MZ + 1] / dn
        c = cfg.coll * dn
        vx2, vy2, vz2 = v ** 2
        s[PXX] = c * (2 * vx2 - vy2 - vz2) / 3
        s[PYY] = c * (2 * vy2 - vz2 - vx2) / 3
        s[PZZ] = c * (2 * vz2 - vx2 - vy2) / 3
        s[PXY], s[PXZ], s[PYZ] = c * v[0] * v[1], c * v[0] * v[2], c * v[1] * v[2]
    return s


def state(rng, ivis, rho, vel, p, g, stress=0.1):
    q = np.zeros(11)
    vel = np.asarray(vel, dtype=float)
    q[RH] = rho
    q[MX:MZ + 1] = rho * vel
    q[EN] = p / (g - 1) + 0.5 * rho * vel @ vel
    dev = rng.uniform(-stress, stress, 6)
    if ivis == 2:                              # full second moments rho v v + p I + deviation
        for (a, b), k in (((0, 0), PXX), ((1, 1), PYY), ((2, 2), PZZ), ((0, 1), PXY), ((0, 2), PXZ), ((1, 2), PYZ)):
            q[k] = rho * vel[a] * vel[b] + (p if a == b else 0.0) + dev[k - PXX]
    else:
        q[PXX:] = dev
    return q


def line_config(d, **kw):
    n = [1, 1, 1]
    n[d] = 3
    ln = [0.5, 0.5, 0.5]
    ln[d] = 1.5
    return config.Config(nx=n[0], ny=n[1], nz=n[2], nbasis=4, iquad=2, iorder=2, lx=ln[0], ly=ln[1], lz=ln[2], **kw)


def compare(cfg, d, states, stale=True):
    import oracle as O
    Q = np.zeros(cfg.shape_f, order="F")
    for i, q in enumerate(states):
        idx = [0, 0, 0]
        idx[d] = i
        Q[idx[0], idx[1], idx[2], :, 0] = q
    r = O.Oracle(cfg).rhs(Q, limit=False)
    dxi = 3 / [cfg.lx, cfg.ly, cfg.lz][d]
    waves = []
    for i in range(3):
        F_hi, w = face_flux(cfg, states[i], states[(i + 1) % 3], d, stale)
        F_lo, _ = face_flux(cfg, states[(i - 1) % 3], states[i], d, stale)
        waves.append(w)
        want = dxi * (F_hi - F_lo) - source(cfg, states[i])
        idx = [0, 0, 0]
        idx[d] = i
        got = r[idx[0], idx[1], idx[2], :, 0]
        scale = max(1.0, np.abs(want).max())
        assert np.abs(got - want).max() <= 1e-13 * scale, (d, i, got - want)
    return waves


@pytest.mark.parametrize("d", [0, 1, 2])
@pytest.mark.parametrize("ivis,ieos,ihllc", [(0, 1, 1), (1, 1, 1), (2, 1, 1), (0, 1, 0), (2, 1, 0), (0, 2, 1),
                                             (1, 2, 0), (0, 1, 2), (1, 1, 2), (2, 1, 2)])
def test_random_states(d, ivis, ieos, ihllc):
    rng = np.random.default_rng(100 * d + 10 * ivis + 3 * ieos + ihllc)
    cfg = line_config(d, ivis=ivis, ieos=ieos, ihllc=ihllc, coll=0.7 if ivis != 1 else 0.0, colvis=0.3,
                      P_1=0.05, P_base=1.0)
    for _ in range(4):
        states = [state(rng, ivis, rng.uniform(0.5, 2.0), rng.uniform(-1.0, 1.0, 3), rng.uniform(0.5, 2.0),
                        cfg.aindex) for _ in range(3)]
        compare(cfg, d, states)


@pytest.mark.parametrize("d", [0, 1, 2])
def test_hllc_branches_and_tie(d):
    """States that put every face on a given HLLC branch: supersonic either way
    (F_L, F_R), subsonic with the contact moving either way (F_L*, F_R*), and
    mirror states whose contact speed is exactly zero (the reference's later
    test takes F_R*)."""
    rng = np.random.default_rng(7 + d)
    cfg = line_config(d, ivis=1, ieos=1, ihllc=1, coll=0.0, colvis=0.2)
    g = cfg.aindex
    e = np.eye(3)[d]
    seen = set()

    def branch(w):
        SL, SM, SR = w
        b = "L" if SL > 0 else "L*" if 0 < SM else "R*" if SR >= 0 else "R"
        return "R" if SR < 0 else b

    cases = {
        "L": [state(rng, 1, r, 4.0 * e, 1.0, g) for r in (1.0, 1.3, 0.8)],
        "R": [state(rng, 1, r, -4.0 * e, 1.0, g) for r in (1.0, 1.3, 0.8)],
        "L*": [state(rng, 1, r, 0.3 * e + 0.2, 1.0, g) for r in (1.0, 1.3, 0.8)],
        "R*": [state(rng, 1, r, -0.3 * e + 0.2, 1.0, g) for r in (1.0, 1.3, 0.8)],
    }
    for name, states in cases.items():
        for w in compare(cfg, d, states):
            seen.add(branch(w))
        assert name in seen, (name, seen)
    # exact tie: equal density and pressure, normal velocities +a | -a
    a = 0.4
    tie = [state(rng, 1, 1.0, a * e, 1.0, g, stress=0.0), state(rng, 1, 1.0, -a * e, 1.0, g, stress=0.0),
           state(rng, 1, 1.0, a * e, 1.0, g, stress=0.0)]
    w = compare(cfg, d, tie)
    assert w[0][1] == 0.0                    # the face between cells 0 and 1 has S_M = 0 exactly


def test_tait_hllc_uses_the_stale_inverse_density():
    """With ieos 2 the reference's sound speeds in HLLC take p * rho_i with
    rho_i = 1/rho of the last point of the call (a right state), not each
    state's own density (flux.f90:513-537): the restatement with the stale
    factor agrees with the oracle, the one with each state's own 1/rho does
    not where the densities differ."""
    cfg = line_config(0, ivis=0, ieos=2, ihllc=1, coll=0.0, colvis=0.0, P_1=0.05, P_base=1.0)
    rng = np.random.default_rng(3)
    states = [state(rng, 0, r, (0.2, 0.0, 0.0), 1.0, cfg.aindex, stress=0.0) for r in (0.6, 1.7, 1.1)]
    compare(cfg, 0, states)
    with pytest.raises(AssertionError):
        compare(cfg, 0, states, stale=False)


@pytest.mark.parametrize("ihllc", [1, 0])
def test_pressure_floor_in_the_point_flux_only(ihllc):
    """A cell whose pressure is half the floor P_floor = T_floor rh_floor
    (params.f90:95): the point flux uses the floored value (flux.f90:62-63),
    HLLC its own unfloored one (flux.f90:513-521)."""
    cfg = line_config(0, ivis=0, ieos=1, ihllc=ihllc, coll=0.0, colvis=0.0)
    pfl = cfg.T_floor * cfg.rh_floor
    rng = np.random.default_rng(11)
    states = [state(rng, 0, 1.0, (0.1, 0.0, 0.0), 1.0, cfg.aindex, stress=0.0),
              state(rng, 0, 0.5, (0.2, 0.0, 0.0), 0.5 * pfl, cfg.aindex, stress=0.0),
              state(rng, 0, 0.8, (0.0, 0.0, 0.0), 0.7, cfg.aindex, stress=0.0)]
    compare(cfg, 0, states)
    f_floor = point_flux(cfg, states[1], 0)
    q_unf = states[1].copy()
    q_unf[EN] += 0.5 * pfl / (cfg.aindex - 1)            # the same state at the floor itself
    assert abs(point_flux(cfg, q_unf, 0)[MX] - f_floor[MX]) < 1e-3 * pfl   # the flux saw the floor

"""The whole time step restated a second time in numpy, against the C oracle:
get_min_dt (hermeshd.f90:145-199), the SSP-RK2/RK3 combinations
(integrator.f90:62-85) of forward-Euler stages that first limit their input
in place (integrator.f90:93-114, so the combination reads the limited state),
and the stage update of each ivis (integrator.f90:125-252; for the Grad
closure, ivis 3, the monolithic 10-moment code's advance_time_level_gl and,
with RK2, its implicit source step after every stage, ten_moment.f90:335-372,
719-892), on top of the
general-form right-hand side of test_oracle_rhs_restatement.py and the numpy
limiter of test_limiter_restatement.py (face-point basis values evaluated here
from the basis definition).  ivis 2 follows the one deviation the oracle
states: the reference never writes rh..en of Q_out in that case, and both
restatements give them the explicit update.

The Tait EOS (ieos 2) runs through the same stages with its own CFL sound
speed sqrt(7.2 P_1 rho^6.2 + T_floor).  Quirks carried: the sound speed sqrt(gamma (E/rho - v^2/2)) with gamma, not
gamma - 1; the maximum over cells with density above rh_mult rh_floor; vmax
adds the LAST cell's sound speed and uses dxi alone; cflm 0.14 (iquad 2) or
0.08 (iquad 3) (initialize.f90:104-122).  Measured: the time bit-identical and
the states within 3e-16 to 6e-16 of each variable's scale after three steps."""
import math

import numpy as np
import pytest

from hermeshd_gb300 import config, ic

from test_limiter_restatement import limiter_numpy
from test_oracle_rhs_restatement import FAMILIES, phi, restated_rhs, rule

RH, MX, MY, MZ, EN, PXX = 0, 1, 2, 3, 4, 5


def min_dt(cfg, Q):
    cflm = cfg.cflm if cfg.cflm > 0 else {2: 0.14, 3: 0.08}[cfg.iquad]
    vmag, cs = 0.0, 0.0
    for k in range(cfg.nz):
        for j in range(cfg.ny):
            for i in range(cfg.nx):
                dn = Q[i, j, k, RH, 0]
                dni = 1.0 / dn
                vx, vy, vz = (Q[i, j, k, m, 0] * dni for m in (MX, MY, MZ))
                if cfg.ieos == 1:
                    cs = math.sqrt(cfg.aindex * (Q[i, j, k, EN, 0] * dni - 0.5 * (vx ** 2 + vy ** 2 + vz ** 2)))
                else:
                    cs = math.sqrt(7.2 * cfg.P_1 * dn ** 6.2 + cfg.T_floor)
                v0 = max(abs(vx) + cs, abs(vy) + cs, abs(vz) + cs)
                if v0 > vmag and dn > 1.01 * cfg.rh_floor:
                    vmag = v0
    return cflm / ((vmag + cs) * (cfg.nx / cfg.lx))


def face_basis(cfg):
    """Basis values at the 6 iquad^2 face points (the limiter's edge points)."""
    fams = FAMILIES[cfg.nbasis]
    s, _ = rule(cfg.iquad)
    rows = []
    for d in range(3):
        t1, t2 = [a for a in range(3) if a != d]
        for side in (1.0, -1.0):
            for a in s:
                for c in s:
                    p = [0.0] * 3
                    p[d], p[t1], p[t2] = side, a, c
                    rows.append([phi(f, p) for f in fams])
    return np.array(rows)


def euler_stage(cfg, Q_in, dt, B, step=0, stage=0):
    """Limits Q_in in place, then returns the stage output (the stochastic
    stress of the given step and stage)."""
    Q_in[...] = limiter_numpy(Q_in, cfg, B)
    r = restated_rhs(cfg, Q_in, step, stage)    # glflux - source
    out = Q_in - dt * r
    faci = 1.0 / (1.0 + dt * cfg.coll)
    if cfg.ivis == 1:
        out[..., PXX:, :] *= faci
    elif cfg.ivis == 3 and cfg.iorder == 2:
        # the Grad closure's RK2 follows each advection stage by its implicit
        # source step (ten_moment.f90:342-356,719-892), here on the values
        # before that step (the reference passes one array as both arguments)
        out = grad_source_step(cfg, out, dt)
    elif cfg.ivis == 2:
        P = Q_in[..., PXX:PXX + 3, :]
        g = r[..., PXX:PXX + 3, :]
        # Q_sum - glf_sum + src_sum with r = glflux - source
        extra = cfg.coll * dt * P.sum(axis=-2) / 3 - cfg.coll * dt ** 2 * g.sum(axis=-2) / 3
        out[..., PXX:PXX + 3, :] = faci * (P - dt * g + extra[..., None, :])
        out[..., PXX + 3:, :] *= faci
    return out


def grad_source_step(cfg, Q, dt):
    fams = FAMILIES[cfg.nbasis]
    nb = len(fams)
    cb = [float((2 * a + 1) * (2 * b + 1) * (2 * c + 1)) for a, b, c in fams]
    s, w = rule(cfg.iquad)
    pts = [((s[a], s[b], s[c]), w[a] * w[b] * w[c]) for a in range(len(s)) for b in range(len(s))
           for c in range(len(s))]
    out = Q.copy()
    for i in range(cfg.nx):
        for j in range(cfg.ny):
            for k in range(cfg.nz):
                sr = np.zeros((6, nb))
                for p, wp in pts:
                    ph = np.array([phi(f, p) for f in fams])
                    dn = ph @ Q[i, j, k, RH]
                    vx, vy, vz = (ph @ Q[i, j, k, m] / dn for m in (MX, MY, MZ))
                    c = cfg.coll * dn
                    S = (c * (2 * vx ** 2 - vy ** 2 - vz ** 2) / 3, c * (2 * vy ** 2 - vz ** 2 - vx ** 2) / 3,
                         c * (2 * vz ** 2 - vx ** 2 - vy ** 2) / 3, c * vx * vy, c * vx * vz, c * vy * vz)
                    for m in range(6):
                        sr[m] += 0.125 * np.array(cb) * wp * ph * S[m]
                E = Q[i, j, k, PXX:PXX + 6].copy()
                den = 1.0 + dt * cfg.coll
                esum = cfg.coll * dt * (E[0] + E[1] + E[2]) / 3
                ssum = cfg.coll * dt ** 2 * (sr[0] + sr[1] + sr[2]) / 3
                for m in range(3):
                    out[i, j, k, PXX + m] = (E[m] + dt * sr[m] + esum + ssum) / den
                for m in range(3, 6):
                    out[i, j, k, PXX + m] = (E[m] + dt * sr[m]) / den
    return out


def step(cfg, Q, B, n=0):
    """Step number n (the stochastic stress's step counter; its stage counter
    is the stage's index in the step)."""
    dt = min_dt(cfg, Q)
    q1 = euler_stage(cfg, Q, dt, B, n, 0)
    q2 = euler_stage(cfg, q1, dt, B, n, 1)
    if cfg.iorder == 2:
        return 0.5 * (Q + q2), dt
    q1 = 0.75 * Q + 0.25 * q2
    q2 = euler_stage(cfg, q1, dt, B, n, 2)
    return (1.0 / 3.0) * Q + (2.0 / 3.0) * q2, dt


CASES = [
    # nb, iquad, ivis, ihllc, iorder, y boundaries, ieos
    (4, 2, 0, 1, 2, "periodic", 1),
    (4, 2, 1, 2, 3, "wall", 1),
    (8, 2, 1, 1, 2, "noslip", 1),
    (10, 3, 2, 1, 3, "periodic", 1),
    (10, 3, 0, 0, 3, "wall", 1),
    (4, 2, 0, 1, 2, "wall", 2),
    (10, 3, 1, 1, 3, "periodic", 2),
    (4, 2, 3, 1, 2, "periodic", 1),
    (10, 3, 3, 0, 3, "wall", 1),
    (8, 2, 3, 2, 2, "noslip", 1),
]


@pytest.mark.parametrize("nb,iq,ivis,ihllc,iorder,ybc,ieos", CASES,
                         ids=["nb%d_ivis%d_rk%d_%s%s" % (c[0], c[2], c[4], c[5], "_tait" if c[6] == 2 else "")
                              for c in CASES])
def test_three_steps_match_the_oracle(nb, iq, ivis, ihllc, iorder, ybc, ieos):
    import oracle as O
    cfg = config.Config(nx=3, ny=3, nz=2, nbasis=nb, iquad=iq, ivis=ivis, ieos=ieos, ihllc=ihllc, iorder=iorder,
                        coll=5.0 if ivis != 0 else 0.8, colvis=0.3, lx=1.5, ly=1.2, lz=1.1, ylobc=ybc, yhibc=ybc,
                        P_1=0.05, P_base=1.0)
    Q = ic.random_smooth(cfg, seed=nb + 3 * ivis, amp=0.2, stress_amp=0.05)
    if ivis >= 2:
        ic.ten_moment_stress(cfg, Q, p=1.0, amp=0.05, seed=nb)
    Q = np.asfortranarray(Q)
    B = face_basis(cfg)
    mine, t_mine = Q.copy(), 0.0
    for n in range(3):
        mine, dt = step(cfg, mine, B, n)
        t_mine += dt
    ref = Q.copy(order="F")
    t_ref, dt_ref = O.Oracle(cfg).advance(ref, 3)
    assert abs(t_ref - t_mine) <= 1e-14 * t_ref
    scale = np.abs(ref).max(axis=(0, 1, 2, 4), keepdims=True)
    err = np.abs(ref - mine) / scale
    assert err.max() <= 1e-12, (err.max(), np.unravel_index(err.argmax(), err.shape))
    assert np.abs(ref - Q).max() > 1e-3 * np.abs(Q).max()       # the state moved


def test_limited_state_enters_the_combination():
    """A state the limiter changes: the RK2 combination 0.5 (Q + Q_2) reads
    the LIMITED Q, because the first stage limits its input in place."""
    import oracle as O
    cfg = config.Config(nx=3, ny=2, nz=2, nbasis=4, iquad=2, ivis=0, ieos=1, ihllc=1, iorder=2, coll=0.0,
                        colvis=0.0, lx=1.5, ly=0.8, lz=1.1)
    Q = ic.random_smooth(cfg, seed=4, amp=0.1)
    Q[0, 0, 0, RH, 1:] = 0.9                  # face densities far below zero: theta < 1
    Q = np.asfortranarray(Q)
    B = face_basis(cfg)
    lim = limiter_numpy(Q, cfg, B)
    assert not np.array_equal(lim, Q)
    mine, _ = step(cfg, Q.copy(), B)
    ref = Q.copy(order="F")
    O.Oracle(cfg).advance(ref, 1)
    assert np.abs(ref - mine).max() <= 1e-12 * np.abs(ref).max()
    # combining with the unlimited input instead would differ
    dt = min_dt(cfg, Q)
    q = Q.copy()
    q1 = euler_stage(cfg, q, dt, B)
    q2 = euler_stage(cfg, q1, dt, B)
    assert np.abs(0.5 * (Q + q2) - ref).max() > 1e-6

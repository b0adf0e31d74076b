"""The positivity limiter (flux.f90:1077-1164) restated a second time, in
numpy over whole grids, against the oracle's C restatement on states where it
acts in every branch: a cell average below the density floor, face-point
densities below it (theta on the density modes), an average pressure below
the pressure floor (higher hydro modes zeroed) and face-point pressures below
it (theta on all hydro modes).  Two independent restatements of the same
Fortran agreeing to rounding pin the oracle's limiter."""
import numpy as np
import pytest

from hermeshd_gb300 import config, ic

RH, MX, MY, MZ, EN = 0, 1, 2, 3, 4


def limiter_numpy(Q, cfg, bf_faces):
    """flux.f90:1077-1164 on a Fortran-order Q(nx,ny,nz,nQ,nb) (a copy is returned)."""
    Q = np.array(Q, dtype=np.float64, order="F", copy=True)
    nb = cfg.nbasis
    npge = 6 * cfg.iquad ** 2
    B = bf_faces[:npge, :nb]                                   # face points x basis
    eps, epsP, g1 = cfg.rh_floor, cfg.rh_floor * cfg.T_floor, cfg.aindex - 1.0
    rho0 = Q[..., RH, 0].copy()
    low = rho0 < cfg.rh_floor
    Q[low, RH:EN + 1, 1:] = 0.0
    Q[low, RH, 0] = cfg.rh_floor
    ok = ~low
    # face-point density: theta on the density's higher modes
    rho_e = np.einsum("pb,xyzb->xyzp", B, Q[..., RH, :])
    rmin = rho_e.min(axis=-1)
    lim = ok & (rmin < eps)
    with np.errstate(divide="ignore", invalid="ignore"):
        th = np.clip((eps - rho0) / (rmin - rho0), 0.0, 1.0)
    Q[lim, RH, 1:] *= np.abs(th[lim])[:, None]
    # average pressure from the cell averages
    m2 = Q[..., MX, 0] ** 2 + Q[..., MY, 0] ** 2 + Q[..., MZ, 0] ** 2
    with np.errstate(divide="ignore", invalid="ignore"):
        pave = g1 * (Q[..., EN, 0] - 0.5 * m2 / Q[..., RH, 0])
    zero = ok & (pave < epsP)
    Q[zero, RH:EN + 1, 1:] = 0.0
    rest = ok & ~zero
    # face-point pressures: theta on every hydro mode
    qe = np.einsum("pb,xyzvb->xyzvp", B, Q[..., RH:EN + 1, :])
    with np.errstate(divide="ignore", invalid="ignore"):
        p = g1 * (qe[..., EN, :] - 0.5 / qe[..., RH, :] * (qe[..., MX, :] ** 2 + qe[..., MY, :] ** 2 + qe[..., MZ, :] ** 2))
        pa = pave[..., None]
        thj = np.where((p < epsP) & (pa != p), (pa - epsP) / (pa - p), 1.0)
    th2 = np.clip(np.minimum(1.0, thj.min(axis=-1)), 0.0, 1.0)
    Q[rest, RH:EN + 1, 1:] *= th2[rest][:, None, None]
    return Q


def floored_state(cfg, seed):
    rng = np.random.default_rng(seed)
    Q = ic.random_smooth(cfg, seed=seed, amp=0.05)
    sh = Q[:, :, :, RH, 1:].shape
    Q[:, :, :, RH, 1:] = 0.22 * rng.standard_normal(sh)
    Q[:, :, :, EN, 1:] = 0.25 * rng.standard_normal(sh)
    for v in (MX, MY, MZ):
        Q[:, :, :, v, 1:] = 0.05 * rng.standard_normal(sh)
    Q[0, 0, 0, RH, 0] = 0.35
    m2 = Q[1, 0, 0, MX, 0] ** 2 + Q[1, 0, 0, MY, 0] ** 2 + Q[1, 0, 0, MZ, 0] ** 2
    Q[1, 0, 0, EN, 0] = 0.5 * m2 / Q[1, 0, 0, RH, 0] + 0.1
    return Q


@pytest.mark.parametrize("nb,iq", [(4, 2), (8, 2), (10, 3)])
def test_limiter_restatements_agree(nb, iq):
    import oracle as O
    cfg = config.Config(nx=6, ny=5, nz=3, nbasis=nb, iquad=iq, rh_floor=0.4, T_floor=0.5)
    orc = O.Oracle(cfg)
    bf = orc.table("faces")
    for seed in (3, 4, 5):
        Q = floored_state(cfg, seed)
        ref = np.asfortranarray(Q.copy())
        orc.limiter(ref)
        mine = limiter_numpy(Q, cfg, bf)
        changed = np.any(ref != Q, axis=(3, 4))
        assert changed.sum() >= 10                               # the limiter acted widely
        assert np.allclose(mine, ref, rtol=1e-12, atol=1e-14), float(np.abs(mine - ref).max())
        # every branch was taken somewhere
        assert ref[0, 0, 0, RH, 0] == cfg.rh_floor and not ref[0, 0, 0, RH:EN + 1, 1:].any()
        assert not ref[1, 0, 0, RH:EN + 1, 1:].any()


def test_limiter_leaves_a_smooth_state_alone():
    import oracle as O
    cfg = config.Config(nx=6, ny=5, nz=3, nbasis=8, iquad=2)
    orc = O.Oracle(cfg)
    Q = ic.random_smooth(cfg, seed=1, amp=0.05)
    ref = np.asfortranarray(Q.copy())
    orc.limiter(ref)
    assert np.array_equal(ref, Q)
    assert np.array_equal(limiter_numpy(Q, cfg, orc.table("faces")), Q)

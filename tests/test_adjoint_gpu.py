"""The hand-written adjoint (CUDA VJP kernels + the checkpointed RK adjoint)
against finite differences of the library's own forward map and of the FP64
oracle (the reference's algorithm restated on the CPU).

Tolerances (relative):
  RHS / stage VJP vs central differences              1e-6
  rollout gradient (viscosity, perturbation) vs FD    1e-6
  rollout gradient vs FD of the oracle's rollout      1e-6

States for the operator checks carry a mean flow in every direction, so no
face point sits on a switching surface of the Riemann solvers (HLLC wave
selection, Roe |lambda|), where the forward map is not differentiable.
"""
import numpy as np
import pytest

from hermeshd_gb300 import config, ic
from hermeshd_gb300.config import NQ

pytestmark = pytest.mark.gpu

TOL = 1e-6
RH, MX, MY, MZ, EN = 0, 1, 2, 3, 4


def _torch():
    import torch
    return torch


def generic_state(cfg, seed, mean=(0.9, 0.7, 0.5), stress_amp=0.02):
    """random_smooth plus a uniform mean flow (pressure kept)."""
    Q = ic.random_smooth(cfg, seed=seed, amp=0.05, stress_amp=stress_amp)
    g = cfg.aindex
    rho = Q[:, :, :, RH, 0]
    m = Q[:, :, :, MX:MZ + 1, 0]
    p = (g - 1.0) * (Q[:, :, :, EN, 0] - 0.5 * (m ** 2).sum(-1) / rho)
    for k in range(3):
        Q[:, :, :, MX + k, 0] += rho * mean[k]
    m = Q[:, :, :, MX:MZ + 1, 0]
    Q[:, :, :, EN, 0] = p / (g - 1.0) + 0.5 * (m ** 2).sum(-1) / rho
    return Q


def _direction(q, seed):
    torch = _torch()
    gen = torch.Generator(device=q.device).manual_seed(seed)
    scale = q.abs().mean(dim=(2, 3, 4), keepdim=True) + 1e-3
    return torch.randn(q.shape, generator=gen, dtype=q.dtype, device=q.device) * scale


# (config, seed of the state).  HLLC's wave speeds are min/max of two nearly
# equal values (the two traces of a smooth state), so a state can sit within
# 1e-6 of a kink; the seeds give states whose central differences at h and
# h/10 agree (checked in the test), i.e. no kink within reach of the step.
VJP_CASES = {
    "nb4_3d_periodic_ivis0_hllc": (config.Config(nx=6, ny=5, nz=4, nbasis=4, iquad=2, ivis=0, coll=0.7, lx=1.3,
                                                 ly=0.9, lz=1.1), 8),
    "nb8_3d_ivis1_roe": (config.Config(nx=4, ny=4, nz=3, nbasis=8, iquad=2, ivis=1, coll=3.0, colvis=1.5, ihllc=2), 3),
    "nb10_2d_ivis1_hllc": (config.Config(nx=6, ny=6, nz=1, nbasis=10, iquad=3, ivis=1, coll=2.0, colvis=1.0), 6),
    "nb4_2d_noslip_bodyforce": (config.Config(nx=6, ny=8, nz=1, nbasis=4, iquad=2, ivis=1, coll=5.0, colvis=1.0,
                                              ylobc="noslip", yhibc="noslip", body_force=0.1), 3),
    "nb8_3d_walls_central": (config.Config(nx=5, ny=4, nz=3, nbasis=8, iquad=2, ihllc=0, xlobc="wall", xhibc="wall",
                                           zlobc="noslip", zhibc="wall"), 3),
    "nb4_3d_outflow_y": (config.Config(nx=4, ny=5, nz=3, nbasis=4, iquad=2, ivis=1, coll=1.0, colvis=1.0,
                                       ylobc="outflow", yhibc="outflow"), 8),
}


@pytest.mark.parametrize("name", sorted(VJP_CASES))
def test_rhs_vjp_vs_fd(name):
    from hermeshd_gb300.solver import Solver
    cfg, seed = VJP_CASES[name]
    S = Solver(cfg)
    q = S.from_numpy(generic_state(cfg, seed=seed))

    def fd(V, W, h):
        return float((W * (S.rhs(q + h * V, limit=False) - S.rhs(q - h * V, limit=False))).sum()) / (2 * h)

    for k in range(3):
        V, W = _direction(q, 10 + k), _direction(q, 20 + k)
        adj = float((V * S.rhs_vjp(q, W)).sum())
        f1, f2 = fd(V, W, 1e-6), fd(V, W, 1e-7)
        assert abs(f1 - f2) <= 0.1 * TOL * abs(f1), ("state near a switching surface", name, k, f1, f2)
        assert adj != 0.0
        assert abs(adj - f1) <= TOL * abs(adj), (name, k, adj, f1, abs(adj - f1) / abs(adj))


def test_rhs_vjp_vs_oracle_fd():
    """The FP64 reference gradient: directional derivatives of the oracle's
    right-hand side (the reference's algorithm on the CPU) by central
    differences, against the CUDA VJP."""
    import oracle as O
    from hermeshd_gb300.solver import Solver
    cfg, seed = VJP_CASES["nb4_2d_noslip_bodyforce"]
    S = Solver(cfg)
    orc = O.Oracle(cfg)
    Q = generic_state(cfg, seed=seed)
    q = S.from_numpy(Q)
    V, W = _direction(q, 31), _direction(q, 32)
    adj = float((V * S.rhs_vjp(q, W)).sum())
    Vf, Wf = S.to_numpy(V), S.to_numpy(W)
    h = 1e-6
    rp = orc.rhs(np.asfortranarray(Q + h * Vf), limit=False)
    rm = orc.rhs(np.asfortranarray(Q - h * Vf), limit=False)
    fd = float((Wf * (rp - rm)).sum()) / (2 * h)
    assert abs(adj - fd) <= TOL * abs(adj), (adj, fd)


def test_stage_vjp_and_dcoll_vs_fd():
    from hermeshd_gb300.solver import Solver
    cfg, seed = VJP_CASES["nb4_2d_noslip_bodyforce"]
    S = Solver(cfg)
    q = S.from_numpy(generic_state(cfg, seed=seed))
    dt = 0.2 * S.get_min_dt(q)
    e = S.euler_stage(q.clone(), dt)
    V, W = _direction(q, 41), _direction(q, 42)
    lam_in, dcoll = S.stage_vjp(q, W, dt, e_out=e, want_dcoll=True)
    adj = float((V * lam_in).sum())
    h = 1e-6
    fd = float((W * (S.euler_stage(q + h * V, dt) - S.euler_stage(q - h * V, dt))).sum()) / (2 * h)
    assert abs(adj - fd) <= TOL * abs(adj), (adj, fd)
    hc = 1e-6 * cfg.coll
    Sp, Sm = Solver(cfg.replace(coll=cfg.coll + hc)), Solver(cfg.replace(coll=cfg.coll - hc))
    fdc = float((W * (Sp.euler_stage(q.clone(), dt) - Sm.euler_stage(q.clone(), dt))).sum()) / (2 * hc)
    assert abs(dcoll - fdc) <= TOL * abs(dcoll), (dcoll, fdc)
    # lam_in may alias lam_out
    W2 = W.clone()
    out, _ = S.stage_vjp(q, W2, dt, out=W2)
    assert _torch().equal(out, lam_in)


def _channel(ihllc=2, nx=16, ny=32):
    return config.poiseuille_2d(nx=nx, ny=ny, ihllc=ihllc)


def test_rollout_reproduces_step():
    """RK2 rollout of the adjoint's forward pass == the fused library step, bit for bit."""
    from hermeshd_gb300.adjoint import Rollout
    from hermeshd_gb300.solver import Solver
    cfg = _channel()
    Q = ic.channel(cfg, amplitude=1e-3, seed=0)
    S = Solver(cfg)
    q = S.from_numpy(Q)
    q1 = S.new_state()
    for _ in range(10):
        S.step(q, q1)
    roll = Rollout(cfg)
    qr, _, dts = roll.forward(S.from_numpy(Q), cfg.coll, 10)
    assert _torch().equal(qr, q)
    assert roll.limiter_events == 0


def test_dt_of_matches_kernel():
    from hermeshd_gb300.adjoint import Rollout
    from hermeshd_gb300.solver import Solver
    cfg, seed = VJP_CASES["nb4_3d_periodic_ivis0_hllc"]
    S = Solver(cfg)
    q = S.from_numpy(generic_state(cfg, seed=seed))
    roll = Rollout(cfg)
    assert float(roll.dt_of(q)) == pytest.approx(S.get_min_dt(q), rel=1e-14)


def _loss(roll, cfg, pert, coll, nsteps):
    from hermeshd_gb300.adjoint import channel_state, outflow_kinetic_energy
    q, _, _ = roll.forward(channel_state(cfg, pert), coll, nsteps)
    return float(outflow_kinetic_energy(q, cfg))


# Roe (the channel's flux) and the central flux; HLLC amplifies the channel's
# perturbation (its flux is discontinuous at S_M = 0 with the stress-augmented
# point flux), which leaves nothing smooth to difference.
@pytest.mark.parametrize("ihllc", [2, 0])
def test_rollout_gradient_vs_fd(ihllc):
    torch = _torch()
    from hermeshd_gb300.adjoint import Rollout, channel_perturbation, poiseuille_sensitivities
    cfg = _channel(ihllc=ihllc)
    nsteps, mu, p = 20, 0.05, 1.0
    roll = Rollout(cfg, checkpoint_every=5)
    res = poiseuille_sensitivities(cfg, nsteps=nsteps, viscosity=mu, roll=roll)
    assert res["limiter_events"] == 0
    # viscosity: coll = p / mu
    hm = 1e-4 * mu
    pert = channel_perturbation(cfg)
    Lp = _loss(roll, cfg, pert, p / (mu + hm), nsteps)
    Lm = _loss(roll, cfg, pert, p / (mu - hm), nsteps)
    fd_mu = (Lp - Lm) / (2 * hm)
    assert abs(res["dL_dmu"] - fd_mu) <= TOL * abs(res["dL_dmu"]), (res["dL_dmu"], fd_mu)
    # perturbation field, along a random direction
    gen = torch.Generator(device=pert.device).manual_seed(7)
    D = torch.randn(pert.shape, generator=gen, dtype=pert.dtype, device=pert.device) * 1e-3
    hp = 1e-4
    fd_p = (_loss(roll, cfg, pert + hp * D, p / mu, nsteps) - _loss(roll, cfg, pert - hp * D, p / mu, nsteps)) / (2 * hp)
    adj_p = float((D * res["dL_dpert"]).sum())
    assert abs(adj_p - fd_p) <= TOL * abs(adj_p), (adj_p, fd_p)


def test_rollout_gradient_vs_oracle_fd():
    """dL/dmu against central differences of the oracle's rollout (FP64 CPU
    restatement of the reference's time loop, with its own CFL steps)."""
    import oracle as O
    from hermeshd_gb300.adjoint import Rollout, poiseuille_sensitivities
    cfg = _channel(ihllc=2)
    nsteps, mu, p = 20, 0.05, 1.0
    res = poiseuille_sensitivities(cfg, nsteps=nsteps, viscosity=mu, roll=Rollout(cfg, checkpoint_every=20))

    def L_oracle(m):
        c = cfg.replace(coll=p / m)
        Q = ic.channel(c, amplitude=1e-3, seed=0)
        O.Oracle(c).advance(Q, nsteps)
        ke = 0.5 * (Q[-1, :, :, MX, 0] ** 2 + Q[-1, :, :, MY, 0] ** 2 + Q[-1, :, :, MZ, 0] ** 2) / Q[-1, :, :, RH, 0]
        return ke.sum() * (c.lx / c.nx) * (c.ly / c.ny)

    assert L_oracle(mu) == pytest.approx(res["L"], rel=1e-11)
    hm = 1e-4 * mu
    fd = (L_oracle(mu + hm) - L_oracle(mu - hm)) / (2 * hm)
    assert abs(res["dL_dmu"] - fd) <= TOL * abs(res["dL_dmu"]), (res["dL_dmu"], fd)


def test_checkpoint_interval_invariance():
    from hermeshd_gb300.adjoint import Rollout, poiseuille_sensitivities
    cfg = _channel(ihllc=2)
    a = poiseuille_sensitivities(cfg, nsteps=12, roll=Rollout(cfg, checkpoint_every=1))
    b = poiseuille_sensitivities(cfg, nsteps=12, roll=Rollout(cfg, checkpoint_every=5))
    c = poiseuille_sensitivities(cfg, nsteps=12, roll=Rollout(cfg, checkpoint_every=100))
    assert a["dL_dmu"] == b["dL_dmu"] == c["dL_dmu"]
    assert _torch().equal(a["dL_dpert"], b["dL_dpert"]) and _torch().equal(a["dL_dpert"], c["dL_dpert"])


def test_adjoint_rejects_unsupported():
    from hermeshd_gb300._lib import HermesError
    from hermeshd_gb300.solver import Solver
    cfg = config.Config(nx=4, ny=4, nz=1, nbasis=4, iquad=2, ivis=2, coll=1.0)
    S = Solver(cfg)
    q = S.from_numpy(generic_state(cfg, seed=1))
    with pytest.raises(HermesError):
        S.rhs_vjp(q, q.clone())
    cfg = config.Config(nx=4, ny=4, nz=1, nbasis=4, iquad=2, xlobc="wall", xhibc="periodic")
    S = Solver(cfg)
    q = S.from_numpy(generic_state(cfg, seed=1))
    with pytest.raises(HermesError):
        S.rhs_vjp(q, q.clone())


@pytest.mark.parametrize("name", sorted(VJP_CASES))
def test_reverse_sweep_matches_dual_passes(name, monkeypatch):
    """The point-wise VJPs (numerical face flux; primitives and point fluxes at
    the quadrature points) have two implementations: hand-derived reverse
    sweeps (the default) and forward-mode dual numbers, one pass per input
    column (HERMES_ADJOINT_DUAL=1).  Both are exact derivatives of the same
    maps, so they agree to rounding."""
    from hermeshd_gb300.solver import Solver
    cfg, seed = VJP_CASES[name]
    S = Solver(cfg)
    q = S.from_numpy(generic_state(cfg, seed=seed))
    W = _direction(q, 50)
    monkeypatch.delenv("HERMES_ADJOINT_DUAL", raising=False)
    rev = S.rhs_vjp(q, W)
    dt = 0.2 * S.get_min_dt(q)
    e = S.euler_stage(q.clone(), dt)
    want = cfg.ivis == 1     # dcoll: coll enters the ivis 1 flux through faci
    lam_r, dcoll_r = S.stage_vjp(q, W, dt, e_out=e, want_dcoll=want)
    monkeypatch.setenv("HERMES_ADJOINT_DUAL", "1")
    dual = S.rhs_vjp(q, W)
    lam_d, dcoll_d = S.stage_vjp(q, W, dt, e_out=e, want_dcoll=want)
    scale = float(dual.abs().max())
    assert scale > 0
    assert float((rev - dual).abs().max()) <= 1e-12 * scale
    assert float((lam_r - lam_d).abs().max()) <= 1e-12 * float(lam_d.abs().max())
    if want:
        assert dcoll_r == pytest.approx(dcoll_d, rel=1e-12)

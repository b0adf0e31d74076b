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
    for cfg in (config.Config(nx=4, ny=4, nz=1, nbasis=4, iquad=2, ivis=3, coll=1.0, iorder=2),
                config.Config(nx=4, ny=4, nz=1, nbasis=4, iquad=2, ieos=2, ihllc=1, P_1=0.05, P_base=1.0),
                config.Config(nx=4, ny=4, nz=1, nbasis=4, iquad=2, ivis=1, coll=1.0, colvis=1.0, precision="fp32")):
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


# ---- ivis 2 and the Tait equation of state: one dual pass per column ---------
def _fd_coll(fn, c, W, rel=5e-3):
    """W . d fn / dcoll at c, fn(c) a state, and the estimate's own error
    bound: central differences at h = rel c, h/2 and h/4, pairs combined by
    Richardson extrapolation (error O(h^4)); the estimate is the finer pair's,
    the bound the distance between the two pairs' (it holds the rounding
    noise that remains).  The two states of a difference are subtracted
    element by element before the sum: rows that do not depend on coll then
    cancel exactly, where summing each state first leaves the large rows'
    rounding, ~1e-12 absolute, in the quotient."""
    h = rel * c

    def d(k):
        return float((W * (fn(c + k) - fn(c - k))).sum()) / (2 * k)

    d1, d2, d4 = d(h), d(0.5 * h), d(0.25 * h)
    r1, r2 = (4.0 * d2 - d1) / 3.0, (4.0 * d4 - d2) / 3.0
    return r2, abs(r2 - r1)


def ten_moment_state(cfg, seed):
    """generic_state with the 10-moment stresses P_ij = m_i m_j / rho + p
    delta_ij (+ noise) on the averages and small random higher modes."""
    Q = ic.ten_moment_stress(cfg, generic_state(cfg, seed=seed, stress_amp=0.0), p=1.0, amp=0.01, seed=seed)
    rng = np.random.default_rng(100 + seed)
    for b in range(1, cfg.nbasis):
        Q[:, :, :, 5:, b] = 0.005 * rng.standard_normal(Q[:, :, :, 5:, b].shape)
    return Q


def _state(cfg, seed):
    return ten_moment_state(cfg, seed) if cfg.ivis == 2 else generic_state(cfg, seed=seed)


TAIT = dict(P_1=0.05, P_base=1.0)
GEN_CASES = {
    "nb4_3d_ivis2_hllc": (config.Config(nx=5, ny=4, nz=3, nbasis=4, iquad=2, ivis=2, coll=1.5, colvis=1.0), 1),
    "nb8_2d_ivis2_roe_walls": (config.Config(nx=5, ny=6, nz=1, nbasis=8, iquad=2, ivis=2, coll=0.8, colvis=1.0,
                                             ihllc=2, ylobc="wall", yhibc="noslip"), 2),
    "nb10_2d_ivis2_central": (config.Config(nx=5, ny=5, nz=1, nbasis=10, iquad=3, ivis=2, coll=2.5, colvis=1.0,
                                            ihllc=0), 3),
    "nb4_2d_tait_central": (config.Config(nx=6, ny=5, nz=1, nbasis=4, iquad=2, ieos=2, ihllc=0, coll=0.9, **TAIT), 4),
    "nb10_2d_tait_roe_ivis1": (config.Config(nx=5, ny=5, nz=1, nbasis=10, iquad=3, ieos=2, ihllc=2, ivis=1,
                                             coll=2.0, colvis=1.0, **TAIT), 5),
    "nb8_3d_tait_ivis2_roe": (config.Config(nx=4, ny=4, nz=3, nbasis=8, iquad=2, ieos=2, ihllc=2, ivis=2,
                                            coll=1.2, colvis=1.0, **TAIT), 6),
}


@pytest.mark.parametrize("name", sorted(GEN_CASES))
def test_gen_rhs_vjp_vs_fd(name):
    """The per-column dual passes against central differences of the
    library's own right-hand side."""
    from hermeshd_gb300.solver import Solver
    cfg, seed = GEN_CASES[name]
    S = Solver(cfg)
    q = S.from_numpy(_state(cfg, seed))

    def fd(V, W, h):
        return float((W * (S.rhs(q + h * V, limit=False) - S.rhs(q - h * V, limit=False))).sum()) / (2 * h)

    for k in range(3):
        V, W = _direction(q, 60 + k), _direction(q, 70 + k)
        adj = float((V * S.rhs_vjp(q, W)).sum())
        f1, f2 = fd(V, W, 1e-6), fd(V, W, 1e-7)
        assert abs(f1 - f2) <= 0.1 * TOL * abs(f1), ("state near a switching surface", name, k, f1, f2)
        assert adj != 0.0
        assert abs(adj - f1) <= TOL * abs(adj), (name, k, adj, f1, abs(adj - f1) / abs(adj))


def test_gen_rhs_vjp_vs_oracle_fd():
    """ivis 2 and the Tait EOS against central differences of the oracle's
    right-hand side (the reference's algorithm on the CPU)."""
    import oracle as O
    from hermeshd_gb300.solver import Solver
    for name in ("nb4_3d_ivis2_hllc", "nb4_2d_tait_central"):
        cfg, seed = GEN_CASES[name]
        S = Solver(cfg)
        orc = O.Oracle(cfg)
        Q = _state(cfg, seed)
        q = S.from_numpy(Q)
        V, W = _direction(q, 81), _direction(q, 82)
        adj = float((V * S.rhs_vjp(q, W)).sum())
        Vf, Wf = S.to_numpy(V), S.to_numpy(W)
        h = 1e-6
        rp = orc.rhs(np.asfortranarray(Q + h * Vf), limit=False)
        rm = orc.rhs(np.asfortranarray(Q - h * Vf), limit=False)
        fd = float((Wf * (rp - rm)).sum()) / (2 * h)
        assert abs(adj - fd) <= TOL * abs(adj), (name, adj, fd)


@pytest.mark.parametrize("name", sorted(VJP_CASES))
def test_per_column_passes_match_reverse_sweep(name, monkeypatch):
    """The per-column dual passes (HERMES_ADJOINT_DUAL=2, the path of ivis 2
    and the Tait EOS) reproduce the hand-derived reverse sweeps on the ivis 0/1
    ideal-gas cases to rounding, dcoll included."""
    from hermeshd_gb300.solver import Solver
    cfg, seed = VJP_CASES[name]
    S = Solver(cfg)
    q = S.from_numpy(generic_state(cfg, seed=seed))
    W = _direction(q, 51)
    dt = 0.2 * S.get_min_dt(q)
    e = S.euler_stage(q.clone(), dt)
    monkeypatch.delenv("HERMES_ADJOINT_DUAL", raising=False)
    rev = S.rhs_vjp(q, W)
    lam_r, dc_r = S.stage_vjp(q, W, dt, e_out=e, want_dcoll=True)
    monkeypatch.setenv("HERMES_ADJOINT_DUAL", "2")
    gen = S.rhs_vjp(q, W)
    lam_g, dc_g = S.stage_vjp(q, W, dt, e_out=e, want_dcoll=True)
    assert float((rev - gen).abs().max()) <= 1e-12 * float(gen.abs().max())
    assert float((lam_r - lam_g).abs().max()) <= 1e-12 * float(lam_g.abs().max())
    assert dc_r == pytest.approx(dc_g, rel=1e-11, abs=1e-300)


@pytest.mark.parametrize("name", ["nb4_3d_ivis2_hllc", "nb8_3d_tait_ivis2_roe", "nb4_2d_tait_central",
                                  "nb10_2d_tait_roe_ivis1"])
def test_gen_stage_vjp_and_dcoll_vs_fd(name):
    """Stage VJP (for ivis 2 the factor faci (I + (coll dt/3) J) on the
    diagonal stresses) and lam . dE/dcoll (through the factor and through the
    ivis-2 source) against central differences of the library's stage."""
    from hermeshd_gb300.solver import Solver
    cfg, seed = GEN_CASES[name]
    S = Solver(cfg)
    q = S.from_numpy(_state(cfg, seed))
    dt = 0.2 * S.get_min_dt(q)
    e = S.euler_stage(q.clone(), dt)
    V, W = _direction(q, 91), _direction(q, 92)
    lam_in, dcoll = S.stage_vjp(q, W, dt, e_out=e, want_dcoll=True)
    adj = float((V * lam_in).sum())
    h = 1e-6
    fd = float((W * (S.euler_stage(q + h * V, dt) - S.euler_stage(q - h * V, dt))).sum()) / (2 * h)
    assert abs(adj - fd) <= TOL * abs(adj), (adj, fd)
    if cfg.ivis == 0:   # ieos 2, ivis 0: coll enters only the relaxation source
        assert dcoll != 0.0
    if cfg.coll == 0.0:
        return
    fdc, err = _fd_coll(lambda c: Solver(cfg.replace(coll=c)).euler_stage(q.clone(), dt), cfg.coll, W)
    assert abs(dcoll - fdc) <= TOL * abs(dcoll) + err, (dcoll, fdc, err)


def test_ivis0_dcoll_vs_fd():
    """ivis 0 with the ideal gas: coll enters only the relaxation source
    -coll P of the right-hand side; lam . dE/dcoll = -dt (lam . dR/dcoll)."""
    from hermeshd_gb300.solver import Solver
    cfg, seed = VJP_CASES["nb4_3d_periodic_ivis0_hllc"]
    S = Solver(cfg)
    q = S.from_numpy(generic_state(cfg, seed=seed))
    dt = 0.2 * S.get_min_dt(q)
    e = S.euler_stage(q.clone(), dt)
    W = _direction(q, 93)
    _, dcoll = S.stage_vjp(q, W, dt, e_out=e, want_dcoll=True)
    fdc, err = _fd_coll(lambda c: Solver(cfg.replace(coll=c)).euler_stage(q.clone(), dt), cfg.coll, W)
    assert dcoll != 0.0
    assert abs(dcoll - fdc) <= TOL * abs(dcoll) + err, (dcoll, fdc, err)


@pytest.mark.parametrize("name,iorder", [("nb4_3d_ivis2_hllc", 3), ("nb4_2d_tait_central", 2),
                                         ("nb8_3d_tait_ivis2_roe", 3)])
def test_gen_rollout_gradient_vs_fd(name, iorder):
    """A short rollout (CFL time steps that depend on the state, SSP-RK2 or
    RK3): gradient of L = <W, q_n> in q0 and in coll against central
    differences of the rollout itself."""
    torch = _torch()
    from hermeshd_gb300.adjoint import Rollout, rollout
    from hermeshd_gb300.solver import Solver
    cfg, seed = GEN_CASES[name]
    cfg = cfg.replace(iorder=iorder)
    nsteps = 6
    S = Solver(cfg)
    q0 = S.from_numpy(_state(cfg, seed))
    W = _direction(q0, 94)
    roll = Rollout(cfg, checkpoint_every=4)
    qa = q0.clone().requires_grad_(True)
    ca = torch.tensor(cfg.coll, dtype=torch.float64, device=q0.device, requires_grad=True)
    L = (W * rollout(qa, ca, roll, nsteps)).sum()
    L.backward()
    assert roll.limiter_events == 0

    def loss(q, c):
        qf, _, _ = Rollout(cfg).forward(q, c, nsteps)
        return float((W * qf).sum())

    D = _direction(q0, 95)
    h = 1e-6
    fd_q = (loss(q0 + h * D, cfg.coll) - loss(q0 - h * D, cfg.coll)) / (2 * h)
    adj_q = float((D * qa.grad).sum())
    assert abs(adj_q - fd_q) <= TOL * abs(adj_q), (adj_q, fd_q)
    if cfg.coll > 0:
        # a rollout's dL/dcoll is small against the state: the wider step keeps
        # the rounding noise of the differences below the tolerance
        fd_c, err = _fd_coll(lambda c: Rollout(cfg).forward(q0, c, nsteps)[0], cfg.coll, W, rel=5e-2)
        assert err <= 1e-5 * abs(fd_c)
        assert abs(float(ca.grad) - fd_c) <= TOL * abs(float(ca.grad)) + err, (float(ca.grad), fd_c, err)


# ---- the positivity limiter's active branch ----------------------------------
def limiter_state(cfg, seed):
    """A state on which the limiter (density floor 0.4, pressure floor 0.2)
    acts in many cells through every branch: face-point density below the
    floor (theta of the density), face-point pressure below the floor (theta
    of all hydro slopes), a cell average below the density floor and one with
    the average pressure below the floor."""
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


LIM_FLOORS = dict(rh_floor=0.4, T_floor=0.5)


@pytest.mark.parametrize("nb,iq", [(4, 2), (8, 2), (10, 3)])
def test_limiter_vjp_vs_fd(nb, iq):
    """(dL/dq)^T lam of the limiter against central differences of the
    library's limiter and of the oracle's (flux.f90:1077-1164 on the CPU)."""
    import oracle as O
    torch = _torch()
    from hermeshd_gb300.solver import Solver
    cfg = config.Config(nx=5, ny=4, nz=2, nbasis=nb, iquad=iq, **LIM_FLOORS)
    S = Solver(cfg)
    Q = limiter_state(cfg, 3)
    q = S.from_numpy(Q)
    assert not torch.equal(S.limiter(q.clone()), q)
    V, W = _direction(q, 96), _direction(q, 97)
    lam = S.limiter_vjp(q, W)
    adj = float((V * lam).sum())

    def fd(h):
        return float((W * (S.limiter(q + h * V) - S.limiter(q - h * V))).sum()) / (2 * h)

    f1, f2 = fd(1e-6), fd(1e-7)
    assert abs(f1 - f2) <= 0.1 * TOL * abs(f1), (f1, f2)
    assert abs(adj - f1) <= TOL * abs(adj), (adj, f1)
    orc = O.Oracle(cfg)
    Vf, Wf = S.to_numpy(V), S.to_numpy(W)
    h = 1e-6
    a, b = np.asfortranarray(Q + h * Vf), np.asfortranarray(Q - h * Vf)
    orc.limiter(a)
    orc.limiter(b)
    fo = float((Wf * (a - b)).sum()) / (2 * h)
    assert abs(adj - fo) <= TOL * abs(adj), (adj, fo)
    # stress rows pass through; lam_in may be lam_out
    assert torch.equal(lam[:, 5:], W[:, 5:])
    W2 = W.clone()
    assert torch.equal(S.limiter_vjp(q, W2, out=W2), lam)


def test_rollout_gradient_through_active_limiter_vs_fd():
    """A 3-step RK2 rollout in which the limiter acts in every stage: the
    gradient in q0 against central differences of the rollout."""
    from hermeshd_gb300.adjoint import Rollout, rollout
    from hermeshd_gb300.solver import Solver
    torch = _torch()
    cfg = config.Config(nx=6, ny=5, nz=1, nbasis=4, iquad=2, ihllc=0, coll=0.0, **LIM_FLOORS)
    S = Solver(cfg)
    q0 = S.from_numpy(limiter_state(cfg, 5))
    W = _direction(q0, 98)
    roll = Rollout(cfg, checkpoint_every=2)
    qa = q0.clone().requires_grad_(True)
    L = (W * rollout(qa, torch.tensor(0.0, dtype=torch.float64, device=q0.device), roll, 3)).sum()
    L.backward()
    assert roll.limiter_events >= 6

    def loss(q):
        qf, _, _ = Rollout(cfg).forward(q, 0.0, 3)
        return float((W * qf).sum())

    D = _direction(q0, 99)
    f1 = (loss(q0 + 1e-6 * D) - loss(q0 - 1e-6 * D)) / 2e-6
    f2 = (loss(q0 + 1e-7 * D) - loss(q0 - 1e-7 * D)) / 2e-7
    assert abs(f1 - f2) <= 0.1 * TOL * abs(f1), (f1, f2)
    adj = float((D * qa.grad).sum())
    assert abs(adj - f1) <= TOL * abs(adj), (adj, f1)


# ---- the stochastic stress: pathwise gradients, the realisation held fixed ----
def _fh_cfg(**kw):
    return config.fh_box(4, precision="fp64", seed=11, **kw)


def test_noise_rhs_and_stage_vjp_vs_fd():
    """With the stochastic stress on, the VJPs hold the draw of the context's
    counters fixed (noise step 5, stage 1 or 2) and differentiate the state
    dependence of the stress terms; against central differences of the
    library's right-hand side and stage under the same counters, and
    different from the noise-free VJP by far more than the tolerance."""
    from hermeshd_gb300.solver import Solver
    cfg = _fh_cfg()
    S, S0 = Solver(cfg), Solver(cfg.replace(llns=False))
    q = S.from_numpy(generic_state(cfg, seed=12, stress_amp=0.0))
    V, W = _direction(q, 101), _direction(q, 102)
    S.set_noise_step(5)
    S.set_noise_stage(1)
    adj = float((V * S.rhs_vjp(q, W)).sum())
    f1 = float((W * (S.rhs(q + 1e-6 * V, limit=False) - S.rhs(q - 1e-6 * V, limit=False))).sum()) / 2e-6
    f2 = float((W * (S.rhs(q + 1e-7 * V, limit=False) - S.rhs(q - 1e-7 * V, limit=False))).sum()) / 2e-7
    assert abs(f1 - f2) <= 0.1 * TOL * abs(f1), (f1, f2)
    assert abs(adj - f1) <= TOL * abs(adj), (adj, f1)
    adj0 = float((V * S0.rhs_vjp(q, W)).sum())
    assert abs(adj - adj0) > 100 * TOL * abs(adj), (adj, adj0)
    S.set_noise_stage(2)
    dt = 0.3 * S.get_min_dt(q)
    S.set_noise_step(5)
    lam = S.stage_vjp(q, W, dt)[0]
    adj_s = float((V * lam).sum())
    fs = float((W * (S.euler_stage(q + 1e-6 * V, dt) - S.euler_stage(q - 1e-6 * V, dt))).sum()) / 2e-6
    assert abs(adj_s - fs) <= TOL * abs(adj_s), (adj_s, fs)


@pytest.mark.parametrize("iorder", [2, 3])
def test_noise_rollout_reproduces_step(iorder):
    """The rollout's stages draw the fused step's realisations (noise step n,
    stage index k): with RK2 the same states bit for bit; with RK3, whose
    fused step forms 0.75 q + 0.25 E inside the update kernel, to rounding
    (another draw would differ by the noise amplitude times dt)."""
    from hermeshd_gb300.adjoint import Rollout
    from hermeshd_gb300.solver import Solver
    cfg = _fh_cfg(iorder=iorder)
    Q = ic.equilibrium(cfg)
    S = Solver(cfg)
    q, q1 = S.from_numpy(Q), S.new_state()
    for _ in range(5):
        S.step(q, q1)
    qr, _, _ = Rollout(cfg).forward(S.from_numpy(Q), cfg.coll, 5)
    if iorder == 2:
        assert _torch().equal(qr, q)
    else:
        assert float((qr - q).abs().max()) <= 1e-13 * float(q.abs().max())
        assert float((q - S.from_numpy(Q)).abs().max()) > 1e-6   # the noise moved the state


def test_noise_rollout_gradient_vs_fd():
    """Pathwise gradient of a 4-step RK2 rollout with the stochastic stress
    in q0 and in coll against central differences of the rollout under the
    same realisations."""
    torch = _torch()
    from hermeshd_gb300.adjoint import Rollout, rollout
    from hermeshd_gb300.solver import Solver
    cfg = _fh_cfg()
    S = Solver(cfg)
    q0 = S.from_numpy(generic_state(cfg, seed=13, stress_amp=0.0))
    W = _direction(q0, 103)
    roll = Rollout(cfg, checkpoint_every=3)
    qa = q0.clone().requires_grad_(True)
    ca = torch.tensor(cfg.coll, dtype=torch.float64, device=q0.device, requires_grad=True)
    (W * rollout(qa, ca, roll, 4)).sum().backward()

    def loss(q, c):
        qf, _, _ = Rollout(cfg).forward(q, c, 4)
        return float((W * qf).sum())

    D = _direction(q0, 104)
    f1 = (loss(q0 + 1e-6 * D, cfg.coll) - loss(q0 - 1e-6 * D, cfg.coll)) / 2e-6
    adj = float((D * qa.grad).sum())
    assert abs(adj - f1) <= TOL * abs(adj), (adj, f1)
    fc, err = _fd_coll(lambda c: Rollout(cfg).forward(q0, c, 4)[0], cfg.coll, W)
    assert err <= 1e-5 * abs(fc)
    assert abs(float(ca.grad) - fc) <= TOL * abs(float(ca.grad)) + err, (float(ca.grad), fc, err)


def test_argument_checks_of_the_new_entry_points():
    """hermes_set_noise_stage takes 0..2; hermes_limiter_vjp rejects lam_in
    aliasing q; both leave the context usable."""
    from hermeshd_gb300._lib import HermesError
    from hermeshd_gb300.solver import Solver
    cfg = _fh_cfg()
    S = Solver(cfg)
    for bad in (-1, 3):
        with pytest.raises(HermesError):
            S.set_noise_stage(bad)
    S.set_noise_stage(2)
    q = S.from_numpy(generic_state(cfg, seed=1, stress_amp=0.0))
    with pytest.raises(HermesError):
        S.limiter_vjp(q, q.clone(), out=q)
    W = _direction(q, 5)
    assert _torch().equal(S.limiter_vjp(q, W), W)   # no floor within reach: the identity

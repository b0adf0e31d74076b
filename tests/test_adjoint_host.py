"""Host-side pieces of the adjoint, on the CPU: the differentiable CFL time
step against the oracle's get_min_dt, and the torch channel initial state
against ic.channel."""
import numpy as np
import pytest

from hermeshd_gb300 import config, ic


def test_dt_of_matches_oracle():
    torch = pytest.importorskip("torch")
    import oracle as O
    from hermeshd_gb300.adjoint import Rollout
    cfg = config.Config(nx=6, ny=5, nz=4, nbasis=4, iquad=2, ivis=1, coll=2.0, colvis=1.0)
    Q = ic.random_smooth(cfg, seed=2, amp=0.1)
    q = torch.from_numpy(np.ascontiguousarray(Q.T))
    dt = float(Rollout(cfg).dt_of(q))
    assert dt == pytest.approx(O.Oracle(cfg).get_min_dt(Q), rel=1e-14)


def test_dt_of_gradient_is_local():
    """d dt / dq touches only the cell averages of the arg-max cell and the last cell."""
    torch = pytest.importorskip("torch")
    from hermeshd_gb300.adjoint import Rollout
    cfg = config.Config(nx=5, ny=4, nz=3, nbasis=4, iquad=2)
    Q = ic.random_smooth(cfg, seed=3, amp=0.1)
    q = torch.from_numpy(np.ascontiguousarray(Q.T)).requires_grad_(True)
    dt = Rollout(cfg).dt_of(q)
    (g,) = torch.autograd.grad(dt, q)
    nz = torch.nonzero(g)
    assert set(nz[:, 0].tolist()) == {0}          # basis 0 only
    assert set(nz[:, 1].tolist()) <= {0, 1, 2, 3, 4}
    cells = {tuple(r) for r in nz[:, 2:].tolist()}
    assert 1 <= len(cells) <= 2 and (cfg.nz - 1, cfg.ny - 1, cfg.nx - 1) in cells
    # FD check of the smooth map
    h = 1e-7
    d = torch.zeros_like(q)
    d[0, :5] = torch.randn(d[0, :5].shape, dtype=q.dtype)
    roll = Rollout(cfg)
    fd = (float(roll.dt_of(q.detach() + h * d)) - float(roll.dt_of(q.detach() - h * d))) / (2 * h)
    assert fd == pytest.approx(float((g * d).sum()), rel=1e-6)


def test_channel_state_matches_ic():
    torch = pytest.importorskip("torch")
    from hermeshd_gb300.adjoint import channel_perturbation, channel_state
    cfg = config.poiseuille_2d(nx=8, ny=12)
    pert = channel_perturbation(cfg, amplitude=1e-3, seed=0, device=torch.device("cpu"))
    q = channel_state(cfg, pert)
    Q = ic.channel(cfg, amplitude=1e-3, seed=0)
    assert np.array_equal(q.numpy(), np.ascontiguousarray(Q.T))


def test_dt_grad_closed_form_equals_full_autograd():
    """The closed-form d dt / dq of the backward pass (no host synchronisation)
    against autograd through the whole CFL reduction; including a state whose
    arg-max cell is the last cell."""
    torch = pytest.importorskip("torch")
    from hermeshd_gb300.adjoint import Rollout
    for seed in (3, 4, 5):
        cfg = config.Config(nx=5, ny=4, nz=3, nbasis=4, iquad=2)
        Q = ic.random_smooth(cfg, seed=seed, amp=0.1)
        if seed == 5:   # fastest cell = last cell
            Q[-1, -1, -1, 1, 0] += 0.5 * Q[-1, -1, -1, 0, 0]
        q = torch.from_numpy(np.ascontiguousarray(Q.T))
        r = Rollout(cfg)
        a = q.clone().requires_grad_(True)
        dt = r.dt_of(a)
        (g_ref,) = torch.autograd.grad(dt, a)
        g = r._dt_grad(q, float(dt.detach()))
        assert torch.count_nonzero(g) == torch.count_nonzero(g_ref)
        assert torch.allclose(g, g_ref, rtol=1e-13, atol=0.0)


def _tait_cfg():
    return config.Config(nx=5, ny=4, nz=3, nbasis=4, iquad=2, ieos=2, ihllc=2, P_1=0.05, P_base=1.0)


def test_dt_of_tait_matches_oracle():
    """The CFL step with the Tait sound speed 7.2 P_1 rho^6.2 + T_floor
    (hermeshd.f90:166) against the oracle's get_min_dt."""
    torch = pytest.importorskip("torch")
    import oracle as O
    from hermeshd_gb300.adjoint import Rollout
    cfg = _tait_cfg()
    Q = ic.random_smooth(cfg, seed=6, amp=0.1)
    q = torch.from_numpy(np.ascontiguousarray(Q.T))
    assert float(Rollout(cfg).dt_of(q)) == pytest.approx(O.Oracle(cfg).get_min_dt(Q), rel=1e-14)


def test_dt_grad_tait_closed_form_equals_full_autograd():
    torch = pytest.importorskip("torch")
    from hermeshd_gb300.adjoint import Rollout
    cfg = _tait_cfg()
    for seed in (3, 4):
        Q = ic.random_smooth(cfg, seed=seed, amp=0.1)
        if seed == 4:   # fastest cell = last cell
            Q[-1, -1, -1, 1, 0] += 0.5 * Q[-1, -1, -1, 0, 0]
        q = torch.from_numpy(np.ascontiguousarray(Q.T))
        r = Rollout(cfg)
        a = q.clone().requires_grad_(True)
        dt = r.dt_of(a)
        (g_ref,) = torch.autograd.grad(dt, a)
        g = r._dt_grad(q, float(dt.detach()))
        assert torch.count_nonzero(g) == torch.count_nonzero(g_ref)
        assert torch.allclose(g, g_ref, rtol=1e-13, atol=0.0)


def test_ddt_stage_ivis2_matches_autograd():
    """lam . dE/ddt of an ivis-2 stage, E = M(dt) (x - dt R) with R held
    fixed: the closed form of the backward pass against autograd through M."""
    torch = pytest.importorskip("torch")
    from hermeshd_gb300.adjoint import Rollout
    cfg = config.Config(nx=3, ny=2, nz=2, nbasis=4, iquad=2, ivis=2, coll=1.7, colvis=1.0)
    g = torch.Generator().manual_seed(0)
    x = torch.randn(cfg.shape_c, generator=g, dtype=torch.float64)
    R = torch.randn(cfg.shape_c, generator=g, dtype=torch.float64)
    lam = torch.randn(cfg.shape_c, generator=g, dtype=torch.float64)
    coll = cfg.coll

    def stage(dt):
        y = x - dt * R
        faci = 1.0 / (1.0 + dt * coll)
        e = y.clone()
        e[:, 5:] = faci * y[:, 5:]
        d = y[:, 5:8]
        e[:, 5:8] = faci * (d + (coll * dt / 3.0) * d.sum(1, keepdim=True))
        return e

    dt0 = 0.013
    dt = torch.tensor(dt0, dtype=torch.float64, requires_grad=True)
    (ref,) = torch.autograd.grad((lam * stage(dt)).sum(), dt)
    got = Rollout(cfg)._ddt_stage(x, stage(torch.tensor(dt0, dtype=torch.float64)).detach(), lam, dt0, coll)
    assert float(got) == pytest.approx(float(ref), rel=1e-12)

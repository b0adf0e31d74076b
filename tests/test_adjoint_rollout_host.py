"""The adjoint's host-side composition on the CPU: Rollout's forward, its
checkpointed backward (segment recomputation, the SSP-RK2/RK3 transposes, the
limiter and stage VJPs in the right order, the CFL time step's gradient, the
collision frequency's gradient through the stage factor and the right-hand
side) against torch autograd through the same time loop.

The stage operators are a stand-in solver written in torch with the
library's structure -- a limiter applied in place to each stage input, then
E = M (x - dt R(x)) with R independent of dt, coll inside R for ivis 0 and 2,
and M the semi-implicit stress factor of each ivis (integrator.f90:137-224) --
and their VJPs taken by autograd, so any error in how Rollout assembles them
shows up as a mismatch with autograd of the whole loop.  (The CUDA VJP
kernels themselves are checked against finite differences on the GPU.)"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from hermeshd_gb300 import adjoint, config, ic  # noqa: E402

PXX, PZZ = 5, 7


class FakeSolver:
    def __init__(self, roll, coll):
        self.roll, self.coll, self.cfg = roll, float(coll), roll.cfg.replace(coll=float(coll))

    # the operators, differentiable in x and coll
    def lim(self, x):
        y = x.clone()
        y[1:] = x[1:] - 0.02 * torch.tanh(x[1:])
        return y

    def R(self, x, coll):
        r = 0.3 * (x - x.roll(1, -1)) + 0.2 * (x - x.roll(-1, -2)) + 0.05 * torch.sin(x)
        r = r + 0.1 * x[:, :1] * torch.tanh(x.roll(1, 0))
        if self.cfg.ivis == 0:
            r[:, PXX:] = r[:, PXX:] + coll * x[:, PXX:]                              # relaxation -coll P
        elif self.cfg.ivis == 2:
            r[:, PXX:] = r[:, PXX:] - coll * 0.3 * torch.tanh(x[:, :1] * x[:, 1:2]) * x[:, PXX:]
        return r

    def M(self, y, dt, coll):
        iv = self.cfg.ivis
        if iv == 0:
            return y
        faci = 1.0 / (1.0 + dt * coll)
        out = y.clone()
        out[:, PXX:] = faci * y[:, PXX:]
        if iv == 2:
            yd = y[:, PXX:PZZ + 1]
            out[:, PXX:PZZ + 1] = faci * (yd + (coll * dt / 3.0) * yd.sum(1, keepdim=True))
        return out

    def E(self, x, dt, coll):
        return self.M(x - dt * self.R(x, coll), dt, coll)

    # the Solver interface Rollout uses
    def get_min_dt(self, q):
        return float(self.roll.dt_of(q))

    def set_noise_step(self, n):
        pass

    def set_noise_stage(self, k):
        pass

    def euler_stage(self, x, dt):
        with torch.no_grad():
            x.copy_(self.lim(x))
            return self.E(x, dt, self.coll)

    # (these run inside the autograd Function's backward, where grad mode is off)
    def stage_vjp(self, x, lam, dt, e_out=None, want_dcoll=False):
        with torch.enable_grad():
            xx = x.detach().clone().requires_grad_(True)
            c = torch.tensor(self.coll, dtype=torch.float64, requires_grad=True)
            gx, gc = torch.autograd.grad((lam * self.E(xx, dt, c)).sum(), [xx, c])
        return gx, (gc.detach() if want_dcoll else None)

    def limiter_vjp(self, xr, lam, out=None):
        with torch.enable_grad():
            xx = xr.detach().clone().requires_grad_(True)
            (g,) = torch.autograd.grad((lam * self.lim(xx)).sum(), [xx])
        if out is not None:
            out.copy_(g)
            return out
        return g


def reference_loop(roll, fake, q0, coll, nsteps):
    """The same time loop, differentiable end to end (dt included)."""
    q = q0
    for _ in range(nsteps):
        dt = roll.dt_of(q)

        def stage(xr):
            x = fake.lim(xr)
            return x, fake.E(x, dt, coll)
        x0, e1 = stage(q)
        x1, e2 = stage(e1)
        if roll.cfg.iorder == 2:
            q = 0.5 * (x0 + e2)
        else:
            x2, e3 = stage(0.75 * x0 + 0.25 * e2)
            q = (1.0 / 3.0) * x0 + (2.0 / 3.0) * e3
    return q


@pytest.mark.parametrize("ivis,iorder,every", [(1, 2, 2), (1, 3, 3), (0, 3, 2), (2, 2, 1), (2, 3, 4)])
def test_rollout_gradients_equal_autograd_of_the_loop(ivis, iorder, every):
    cfg = config.Config(nx=4, ny=3, nz=2, nbasis=4, iquad=2, ivis=ivis, iorder=iorder, coll=1.3, colvis=0.5,
                        lx=1.0, ly=0.75, lz=0.5)
    roll = adjoint.Rollout(cfg, checkpoint_every=every)
    fakes = {}
    roll.solver = lambda c: fakes.setdefault(float(c), FakeSolver(roll, c))
    Q = ic.random_smooth(cfg, seed=3, amp=0.05, stress_amp=0.02)
    if ivis == 2:
        ic.ten_moment_stress(cfg, Q, p=1.0, amp=0.02, seed=1)
    q0 = torch.from_numpy(np.ascontiguousarray(Q.T))
    w = torch.from_numpy(np.random.default_rng(5).standard_normal(tuple(q0.shape)))
    nsteps = 5

    qa = q0.clone().requires_grad_(True)
    ca = torch.tensor(cfg.coll, dtype=torch.float64, requires_grad=True)
    La = (w * adjoint.rollout(qa, ca, roll, nsteps)).sum()
    La.backward()

    qr = q0.clone().requires_grad_(True)
    cr = torch.tensor(cfg.coll, dtype=torch.float64, requires_grad=True)
    fake = FakeSolver(roll, cfg.coll)
    Lr = (w * reference_loop(roll, fake, qr, cr, nsteps)).sum()
    gq, gc = torch.autograd.grad(Lr, [qr, cr])

    La, Lr = float(La.detach()), float(Lr.detach())
    assert abs(La - Lr) <= 1e-13 * abs(Lr)                                # the forward is the same loop
    assert torch.allclose(qa.grad, gq, rtol=1e-10, atol=1e-13 * gq.abs().max()), \
        float((qa.grad - gq).abs().max() / gq.abs().max())
    assert abs(float(ca.grad) - float(gc)) <= 1e-10 * abs(float(gc)), (float(ca.grad), float(gc))
    # the time step's gradient is part of it: without it the two differ
    lam0, _ = roll.backward(cfg.coll, {0: q0.clone()}, [fake.get_min_dt(q0)], w, with_dt=False)
    qr1 = q0.clone().requires_grad_(True)
    (g1,) = torch.autograd.grad((w * reference_loop(roll, fake, qr1, cr.detach(), 1)).sum(), [qr1])
    assert (lam0 - g1).abs().max() > 1e-9 * g1.abs().max()

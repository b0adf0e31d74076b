"""Hand-written adjoint of the SSP-RK time loop behind torch.autograd.Function.

The forward map is the library's time loop on one FP64 grid: each step takes
dt from the CFL reduction of the cell averages (hermeshd.f90:145-199,
``Solver.get_min_dt``) and runs the SSP-RK stages of integrator.f90:62-86,
each stage the library's forward-Euler stage E(q) = M (q - dt R(q)) with M the
semi-implicit stress factor faci = 1/(1 + dt coll) of ivis 1
(integrator.f90:174).  For RK2 the stages and combinations are the same
operations, in the same order, as the fused ``Solver.step``, so the rollout
reproduces it bit for bit.

The backward pass is the transpose, step by step in reverse:

* each stage's vector-Jacobian product comes from the CUDA adjoint kernels
  (``Solver.stage_vjp``): Riemann flux, volume and surface quadrature,
  sources and the stress factor;
* the RK combinations are linear;
* the time step depends on the state: dL/ddt is the sum over stages of
  lam . dE/ddt, with dE/ddt = (E - M q)/dt, minus coll faci E on the ivis-1
  stresses, and dt = cflm / ((vmag + cs_last) dxi) is differentiated through
  its maximum (the arg-max cell) and the last cell's sound speed;
* the collision frequency coll (for ivis 1 the viscosity enters only as
  coll = p/mu, since colvis = p) through faci.

The positivity limiter is treated as the identity; the forward pass counts
the stages in which it changed the state (``Rollout.limiter_events``), so a
gradient taken where it acted is flagged.

Checkpointing: the forward keeps the state every ``checkpoint_every`` steps;
the backward recomputes each segment's stage states from its checkpoint, one
extra forward pass in total, holding one segment's stage states at a time.
"""
from __future__ import annotations

import math
import warnings
from typing import Dict, List, Optional, Tuple

from .config import NQ, Config
from .solver import Solver

RH, MX, MY, MZ, EN, PXX = 0, 1, 2, 3, 4, 5


def _torch():
    import torch
    return torch


class Rollout:
    """Differentiable n-step rollout of one FP64 problem."""

    def __init__(self, cfg: Config, checkpoint_every: int = 20, check_limiter: bool = True):
        if cfg.precision != "fp64":
            raise ValueError("the adjoint runs in FP64")
        if cfg.ivis not in (0, 1) or cfg.ieos != 1 or cfg.llns:
            raise ValueError("the adjoint supports ivis 0/1, ieos 1, no stochastic stress")
        if cfg.iorder not in (2, 3):
            raise ValueError("iorder must be 2 or 3")
        self.cfg = cfg
        self.checkpoint_every = max(1, int(checkpoint_every))
        self.check_limiter = check_limiter
        self.limiter_events = 0
        self._solvers: Dict[float, Solver] = {}

    def solver(self, coll: float) -> Solver:
        key = float(coll)
        s = self._solvers.get(key)
        if s is None:
            s = Solver(self.cfg.replace(coll=key))
            self._solvers[key] = s
        return s

    # ---- forward ------------------------------------------------------------
    def _stage(self, S: Solver, x, dt: float, check: bool):
        if check:
            x0 = x.clone()
            e = S.euler_stage(x, dt)
            if not _torch().equal(x, x0):
                self.limiter_events += 1
            return e
        return S.euler_stage(x, dt)

    def step(self, S: Solver, q, dt: float, check: Optional[bool] = None) -> Tuple[object, List[Tuple[object, object]]]:
        """One step at a given dt; returns (q_new, [(stage input, E(input))]).
        check: count the stages the limiter changed (default: check_limiter;
        the backward pass's recomputation skips it, the forward counted)."""
        ck = self.check_limiter if check is None else check
        if self.cfg.iorder == 2:
            e1 = self._stage(S, q, dt, ck)
            e2 = self._stage(S, e1, dt, ck)
            return 0.5 * (q + e2), [(q, e1), (e1, e2)]
        e1 = self._stage(S, q, dt, ck)
        e2 = self._stage(S, e1, dt, ck)
        x2 = 0.75 * q + 0.25 * e2
        e3 = self._stage(S, x2, dt, ck)
        return (1.0 / 3.0) * q + (2.0 / 3.0) * e3, [(q, e1), (e1, e2), (x2, e3)]

    def forward(self, q0, coll: float, nsteps: int):
        """Returns (q_final, checkpoints {step: state}, dts)."""
        S = self.solver(coll)
        q = q0.detach().clone().contiguous()
        ckpts = {0: q.clone()}
        dts: List[float] = []
        for n in range(nsteps):
            dt = S.get_min_dt(q)
            q, _ = self.step(S, q, dt)
            dts.append(dt)
            if (n + 1) % self.checkpoint_every == 0 and n + 1 < nsteps:
                ckpts[n + 1] = q.clone()
        return q, ckpts, dts

    # ---- time step and its derivative --------------------------------------
    def dt_of(self, q):
        """dt of the CFL reduction as a differentiable torch function of the
        cell averages (the arithmetic of the library's k_mindt, ieos 1)."""
        torch = _torch()
        c = self.cfg
        a = q[0, :5]
        rho, mx, my, mz, en = a[0], a[1], a[2], a[3], a[4]
        dni = 1.0 / rho
        vx, vy, vz = mx * dni, my * dni, mz * dni
        cs = torch.sqrt(c.aindex * (en * dni - 0.5 * (vx * vx + vy * vy + vz * vz)))
        v0 = torch.maximum(torch.maximum(vx.abs() + cs, vy.abs() + cs), vz.abs() + cs)
        ok = (v0 > 0) & (rho > c.rh_mult * c.rh_floor)
        vmag = v0[ok].max() if bool(ok.any()) else torch.zeros((), dtype=q.dtype, device=q.device)
        cs_last = cs.reshape(-1)[-1]
        return c.cflm_eff / ((vmag + cs_last) * (c.nx / c.lx))

    def _dt_grad(self, q, dt: float):
        """d dt / dq, on the device without a host synchronisation.

        dt = cflm / ((vmag + cs_last) dxi) depends on the cell averages of the
        arg-max cell of vmag = max_d |v_d| + cs and of the last cell (cs_last):
        d dt = -dt^2 dxi / cflm (d vmag + d cs_last), with, per cell,
        d|v_k| = sgn(v_k) dm_k / rho - |v_k| drho / rho (k the arg-max
        direction) and cs^2 = gamma (E/rho - |v|^2/2)."""
        torch = _torch()
        c = self.cfg
        a = q[0, :5].reshape(5, -1)
        rho, m, en = a[0], a[1:4], a[4]
        v = m / rho
        v2 = (v * v).sum(0)
        cs = torch.sqrt(c.aindex * (en / rho - 0.5 * v2))
        av, k = v.abs().max(0)
        v0 = av + cs
        ok = (v0 > 0) & (rho > c.rh_mult * c.rh_floor)
        imax = torch.argmax(torch.where(ok, v0, torch.full_like(v0, -math.inf)))
        ncell = a.shape[1]
        h = c.aindex / (2.0 * cs * rho)
        gcs = torch.stack([h * (-en / rho + v2), -h * v[0], -h * v[1], -h * v[2], h])   # d cs / d(rho, m, E)
        gv = torch.zeros_like(gcs)
        sg = torch.sign(v.gather(0, k[None])[0])
        gv[0] = -av / rho
        gv.scatter_(0, (k + 1)[None], (sg / rho)[None])
        cells = torch.arange(ncell, device=q.device)
        sel_i = ((cells == imax) & ok.any()).to(q.dtype)
        sel_l = (cells == ncell - 1).to(q.dtype)
        scale = -dt * dt * (c.nx / c.lx) / c.cflm_eff
        g = torch.zeros_like(q)
        g[0, :5] = (scale * (sel_i * (gv + gcs) + sel_l * gcs)).reshape(g[0, :5].shape)
        return g

    def _ddt_stage(self, x, e, lam, dt: float, coll: float):
        """lam . dE/ddt for the stage e = E(x), a 0-d device tensor."""
        g = (e - x) / dt
        if self.cfg.ivis == 1:
            faci = 1.0 / (1.0 + dt * coll)
            es, xs = e[:, PXX:], x[:, PXX:]
            g[:, PXX:] = (es - faci * xs) / dt - coll * faci * es
        return (lam * g).sum()

    def _dcoll_stage(self, e, lam, dt: float, coll: float):
        """lam . dE/dcoll for the stage e = E(x) (ivis 1: the stresses are
        faci (x - dt R) with faci = 1/(1 + dt coll), so dE/dcoll = -dt faci E
        there), a 0-d device tensor."""
        faci = 1.0 / (1.0 + dt * coll)
        return (lam[:, PXX:] * e[:, PXX:]).sum() * (-dt * faci)

    # ---- backward -----------------------------------------------------------
    def step_vjp(self, S: Solver, recs, lam, dt: float, coll: float, with_dt: bool = True):
        """Transpose of one step: (lam_q, dL/dcoll as a 0-d device tensor) from
        lam of its output.  Nothing in it waits for the device."""
        torch = _torch()
        want = self.cfg.ivis == 1
        dcoll = torch.zeros((), dtype=lam.dtype, device=lam.device)
        ddt = torch.zeros((), dtype=lam.dtype, device=lam.device)
        if self.cfg.iorder == 2:
            (x0, e1), (x1, e2) = recs
            lam_e2 = 0.5 * lam
            lam_x1, _ = S.stage_vjp(x1, lam_e2, dt)
            if want:
                dcoll = dcoll + self._dcoll_stage(e2, lam_e2, dt, coll) + self._dcoll_stage(e1, lam_x1, dt, coll)
            if with_dt:
                ddt = ddt + self._ddt_stage(x1, e2, lam_e2, dt, coll) + self._ddt_stage(x0, e1, lam_x1, dt, coll)
            lam_x0, _ = S.stage_vjp(x0, lam_x1, dt)
            lam_x0 += 0.5 * lam
        else:
            (x0, e1), (x1, e2), (x2, e3) = recs
            lam_e3 = (2.0 / 3.0) * lam
            lam_x2, _ = S.stage_vjp(x2, lam_e3, dt)
            lam_e2 = 0.25 * lam_x2
            lam_x1, _ = S.stage_vjp(x1, lam_e2, dt)
            if want:
                dcoll = (dcoll + self._dcoll_stage(e3, lam_e3, dt, coll) + self._dcoll_stage(e2, lam_e2, dt, coll)
                         + self._dcoll_stage(e1, lam_x1, dt, coll))
            if with_dt:
                ddt = (ddt + self._ddt_stage(x2, e3, lam_e3, dt, coll) + self._ddt_stage(x1, e2, lam_e2, dt, coll)
                       + self._ddt_stage(x0, e1, lam_x1, dt, coll))
            lam_x0, _ = S.stage_vjp(x0, lam_x1, dt)
            lam_x0 += (1.0 / 3.0) * lam + 0.75 * lam_x2
        if with_dt:
            lam_x0 += ddt * self._dt_grad(x0, dt)
        return lam_x0, dcoll

    def backward(self, coll: float, ckpts, dts, lam, with_dt: bool = True):
        """(lam_q0, dL/dcoll) from lam of the final state."""
        torch = _torch()
        S = self.solver(coll)
        nsteps = len(dts)
        lam = lam.detach().clone().contiguous()
        dcoll = torch.zeros((), dtype=lam.dtype, device=lam.device)
        for start in sorted(ckpts, reverse=True):
            end = min(start + self.checkpoint_every, nsteps)
            q = ckpts[start].clone()
            seg = []
            for n in range(start, end):
                q, recs = self.step(S, q, dts[n], check=False)
                seg.append(recs)
            for n in range(end - 1, start - 1, -1):
                lam, dc = self.step_vjp(S, seg[n - start], lam, dts[n], coll, with_dt)
                dcoll = dcoll + dc
            del seg
        return lam, float(dcoll)


def _rollout_fn():
    torch = _torch()

    class RolloutFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, q0, coll, roll, nsteps):
            c = float(coll)
            qf, ckpts, dts = roll.forward(q0, c, nsteps)
            ctx.roll, ctx.ckpts, ctx.dts, ctx.coll = roll, ckpts, dts, c
            return qf

        @staticmethod
        def backward(ctx, lam):
            lam0, dcoll = ctx.roll.backward(ctx.coll, ctx.ckpts, ctx.dts, lam)
            if ctx.roll.limiter_events:
                warnings.warn(f"the positivity limiter acted in {ctx.roll.limiter_events} stage(s); "
                              "the adjoint treats it as the identity")
            g = torch.tensor(dcoll, dtype=lam.dtype, device=lam.device)
            return lam0, g, None, None

    return RolloutFn


_FN = None


def rollout(q0, coll, roll: Rollout, nsteps: int):
    """q after nsteps steps from q0, differentiable in q0 and coll (a 0-d
    tensor equal to the collision frequency the steps use)."""
    global _FN
    torch = _torch()
    if _FN is None:
        _FN = _rollout_fn()
    if not isinstance(coll, torch.Tensor):
        coll = torch.tensor(float(coll), dtype=torch.float64, device=q0.device)
    return _FN.apply(q0, coll, roll, nsteps)


# ---- the Poiseuille-channel sensitivity problem --------------------------------
def channel_state(cfg: Config, pert, rho: float = 1.0, p: float = 1.0):
    """Channel at rest plus a velocity perturbation pert = (dvx, dvy), each
    (nz, ny, nx), on the cell averages -- ic.channel as a differentiable
    torch function of the perturbation."""
    torch = _torch()
    q = torch.zeros(cfg.shape_c, dtype=torch.float64, device=pert.device)
    vx, vy = pert[0], pert[1]
    q[0, RH] = rho
    q[0, MX] = rho * vx
    q[0, MY] = rho * vy
    q[0, EN] = p / (cfg.aindex - 1.0) + 0.5 * rho * (vx * vx + vy * vy)
    return q


def channel_perturbation(cfg: Config, amplitude: float = 1.0e-3, seed: int = 0, device=None):
    """The seeded Gaussian perturbation of ic.channel, as a (2, nz, ny, nx) tensor."""
    import numpy as np
    torch = _torch()
    rng = np.random.default_rng(seed)
    sh = (cfg.nx, cfg.ny, cfg.nz)
    vx = amplitude * rng.standard_normal(sh)
    vy = amplitude * rng.standard_normal(sh)
    a = np.stack([vx.T, vy.T])   # (2, nz, ny, nx)
    return torch.from_numpy(np.ascontiguousarray(a)).to(device or torch.device("cuda"))


def outflow_kinetic_energy(q, cfg: Config):
    """Kinetic energy of the cell column at the outflow plane x = lx (the
    periodic x boundary): sum over its cells of |m|^2/(2 rho) of the cell
    averages times the cell area dx dy."""
    a = q[0, :4, :, :, -1]
    ke = 0.5 * (a[1] * a[1] + a[2] * a[2] + a[3] * a[3]) / a[0]
    return ke.sum() * (cfg.lx / cfg.nx) * (cfg.ly / cfg.ny)


def poiseuille_sensitivities(cfg: Config, nsteps: int = 200, viscosity: float = 0.05, p: float = 1.0,
                             amplitude: float = 1.0e-3, seed: int = 0, checkpoint_every: int = 20,
                             roll: Optional[Rollout] = None):
    """Gradient of the outflow kinetic energy after nsteps with respect to the
    viscosity mu (coll = p/mu) and the initial velocity perturbation.
    Returns dict(L, dL_dmu, dL_dpert, limiter_events)."""
    torch = _torch()
    roll = roll or Rollout(cfg, checkpoint_every=checkpoint_every)
    pert = channel_perturbation(cfg, amplitude, seed).requires_grad_(True)
    mu = torch.tensor(viscosity, dtype=torch.float64, device=pert.device, requires_grad=True)
    q0 = channel_state(cfg, pert, p=p)
    qf = rollout(q0, p / mu, roll, nsteps)
    L = outflow_kinetic_energy(qf, cfg)
    L.backward()
    return {"L": float(L.detach()), "dL_dmu": float(mu.grad), "dL_dpert": pert.grad.detach(),
            "limiter_events": roll.limiter_events}

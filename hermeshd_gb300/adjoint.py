"""Hand-written adjoint of the SSP-RK time loop behind torch.autograd.Function.

The forward map is the library's time loop on one FP64 grid: each step takes
dt from the CFL reduction of the cell averages (hermeshd.f90:145-199,
``Solver.get_min_dt``) and runs the SSP-RK stages of integrator.f90:62-86,
each stage the library's forward-Euler stage E(q) = M (q - dt R(q)) with M the
semi-implicit stress factor: faci = 1/(1 + dt coll) on the stresses for ivis 1
(integrator.f90:174), faci on the off-diagonal stresses and
faci (I + (coll dt/3) J) on (pxx, pyy, pzz) for ivis 2 (J the 3x3 matrix of
ones, integrator.f90:207-224).  For RK2 the stages and combinations are the same
operations, in the same order, as the fused ``Solver.step``, so the rollout
reproduces it bit for bit.

The backward pass is the transpose, step by step in reverse:

* each stage's vector-Jacobian product comes from the CUDA adjoint kernels
  (``Solver.stage_vjp``): Riemann flux, volume and surface quadrature,
  sources and the stress factor (ivis 0/1 with the ideal-gas law by
  hand-derived reverse sweeps; ivis 2 and the Tait equation of state, ieos 2,
  by one dual-number pass per column through the forward physics);
* the RK combinations are linear;
* the time step depends on the state: dL/ddt is the sum over stages of
  lam . dE/ddt, with dE/ddt = (dM/ddt) y + M (y - q)/dt, y = M^-1 E, and
  dt = cflm / ((vmag + cs_last) dxi) is differentiated through its maximum
  (the arg-max cell) and the last cell's sound speed (ideal gas or Tait);
* the collision frequency coll: through faci for ivis 1 (the viscosity
  enters only as coll = p/mu, since colvis = p), through the relaxation
  source -coll P of the right-hand side for ivis 0, through both the stage
  factor and the source coll rho (v v - |v|^2/3) for ivis 2.

With the stochastic stress on, the gradient is the pathwise one: step n,
stage k draws the realisation of the library's Philox counters (noise step
noise_step0 + n, stage index k), in the forward pass and again in the
backward pass, which holds it fixed while differentiating the state
dependence of the stress terms (their products with the velocity).

Out of scope: HLLC with ieos 2 (its sound speed takes 1/rho of another face
point, flux.f90:533-534) and ivis 3.

The positivity limiter (flux.f90:1077-1164), applied in place to every stage
input, is differentiated along the branch it takes (``Solver.limiter_vjp``:
the identity where it leaves a cell unchanged; the arg-min face point, the
clamp of theta and the floors as the forward pass took them), so the records
keep each stage input before and after the limiter.  The forward pass counts
the stages in which it acted (``Rollout.limiter_events``): near a switch of
its branch the gradient is one-sided.

Checkpointing: the forward keeps the state every ``checkpoint_every`` steps;
the backward recomputes each segment's stage states from its checkpoint, one
extra forward pass in total, holding one segment's stage states at a time.
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Tuple

from .config import NQ, Config
from .solver import Solver

RH, MX, MY, MZ, EN, PXX, PZZ = 0, 1, 2, 3, 4, 5, 7


def _torch():
    import torch
    return torch


class Rollout:
    """Differentiable n-step rollout of one FP64 problem."""

    def __init__(self, cfg: Config, checkpoint_every: int = 20, check_limiter: bool = True, noise_step0: int = 0):
        """noise_step0: with the stochastic stress on, step n of the rollout
        draws the realisation of noise step noise_step0 + n (stage k of it
        with stage index k, as the library's fused step does)."""
        if cfg.precision != "fp64":
            raise ValueError("the adjoint runs in FP64")
        if cfg.ivis not in (0, 1, 2) or cfg.ieos not in (1, 2):
            raise ValueError("the adjoint supports ivis 0/1/2, ieos 1/2")
        if cfg.ieos == 2 and cfg.ihllc == 1:
            raise ValueError("the adjoint does not take HLLC with ieos 2")
        if cfg.iorder not in (2, 3):
            raise ValueError("iorder must be 2 or 3")
        self.cfg = cfg
        self.checkpoint_every = max(1, int(checkpoint_every))
        self.check_limiter = check_limiter
        self.limiter_events = 0
        self.noise_step0 = int(noise_step0)
        self._solvers: Dict[float, Solver] = {}

    def solver(self, coll: float) -> Solver:
        key = float(coll)
        s = self._solvers.get(key)
        if s is None:
            s = Solver(self.cfg.replace(coll=key))
            self._solvers[key] = s
        return s

    # ---- forward ------------------------------------------------------------
    def _noise(self, S: Solver, n: int, k: Optional[int] = None):
        """Point the context's stochastic-stress counters at stage k of step n."""
        if self.cfg.llns:
            if n is not None:
                S.set_noise_step(self.noise_step0 + n)
            if k is not None:
                S.set_noise_stage(k)

    def _stage(self, S: Solver, xr, dt: float, check: bool, keep: bool, k: int = 0):
        """One forward-Euler stage of the library (limiter in place on its
        input, then E): returns (limited input, E).  keep: xr is left as it
        is (the limiter works on a copy), as the backward pass needs it."""
        self._noise(S, None, k)
        x = xr.clone() if (keep or check) else xr
        e = S.euler_stage(x, dt)
        if check and not _torch().equal(x, xr):
            self.limiter_events += 1
        return x, e

    def step(self, S: Solver, q, dt: float, check: Optional[bool] = None,
             keep: bool = True, n: int = 0) -> Tuple[object, List[Tuple[object, object, object]]]:
        """Step n at a given dt; returns (q_new, [(stage input before the
        limiter, after it, E)]) (the records only with keep; without it q is
        limited in place).  check: count the stages the limiter changed
        (default: check_limiter; the backward pass's recomputation skips it,
        the forward counted)."""
        ck = self.check_limiter if check is None else check
        self._noise(S, n)
        if self.cfg.iorder == 2:
            x0, e1 = self._stage(S, q, dt, ck, keep, 0)
            x1, e2 = self._stage(S, e1, dt, ck, keep, 1)
            return 0.5 * (x0 + e2), ([(q, x0, e1), (e1, x1, e2)] if keep else [])
        x0, e1 = self._stage(S, q, dt, ck, keep, 0)
        x1, e2 = self._stage(S, e1, dt, ck, keep, 1)
        x2r = 0.75 * x0 + 0.25 * e2
        x2, e3 = self._stage(S, x2r, dt, ck, keep, 2)
        return (1.0 / 3.0) * x0 + (2.0 / 3.0) * e3, ([(q, x0, e1), (e1, x1, e2), (x2r, x2, e3)] if keep else [])

    def forward(self, q0, coll: float, nsteps: int):
        """Returns (q_final, checkpoints {step: state}, dts)."""
        S = self.solver(coll)
        q = q0.detach().clone().contiguous()
        ckpts = {0: q.clone()}
        dts: List[float] = []
        for n in range(nsteps):
            dt = S.get_min_dt(q)
            q, _ = self.step(S, q, dt, keep=False, n=n)
            dts.append(dt)
            if (n + 1) % self.checkpoint_every == 0 and n + 1 < nsteps:
                ckpts[n + 1] = q.clone()
        return q, ckpts, dts

    # ---- time step and its derivative --------------------------------------
    def _sound_speed(self, rho, en, v2):
        """The CFL sound speed of the library's k_mindt (hermeshd.f90:165-166):
        gamma (E/rho - |v|^2/2) for the ideal gas, 7.2 P_1 rho^6.2 + T_floor
        for the Tait equation of state."""
        torch = _torch()
        c = self.cfg
        if c.ieos == 2:
            return torch.sqrt(7.2 * c.P_1 * torch.pow(rho, 6.2) + c.T_floor)
        return torch.sqrt(c.aindex * (en / rho - 0.5 * v2))

    def dt_of(self, q):
        """dt of the CFL reduction as a differentiable torch function of the
        cell averages (the arithmetic of the library's k_mindt)."""
        torch = _torch()
        c = self.cfg
        a = q[0, :5]
        rho, mx, my, mz, en = a[0], a[1], a[2], a[3], a[4]
        dni = 1.0 / rho
        vx, vy, vz = mx * dni, my * dni, mz * dni
        if c.ieos == 2:
            cs = self._sound_speed(rho, en, None)
        else:
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
        direction) and cs^2 = gamma (E/rho - |v|^2/2) (ideal gas) or
        7.2 P_1 rho^6.2 + T_floor (Tait)."""
        torch = _torch()
        c = self.cfg
        a = q[0, :5].reshape(5, -1)
        rho, m, en = a[0], a[1:4], a[4]
        v = m / rho
        v2 = (v * v).sum(0)
        cs = self._sound_speed(rho, en, v2)
        av, k = v.abs().max(0)
        v0 = av + cs
        ok = (v0 > 0) & (rho > c.rh_mult * c.rh_floor)
        imax = torch.argmax(torch.where(ok, v0, torch.full_like(v0, -math.inf)))
        ncell = a.shape[1]
        if c.ieos == 2:
            z = torch.zeros_like(cs)
            gcs = torch.stack([7.2 * 6.2 * c.P_1 * torch.pow(rho, 5.2) / (2.0 * cs), z, z, z, z])
        else:
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
        """lam . dE/ddt for the stage e = E(x), a 0-d device tensor.

        E = M y, y = x - dt R(x): dE/ddt = (dM/ddt) y + M (y - x)/dt
        = (E - M x)/dt + (dM/ddt) y.  ivis 1: M = faci on the stresses,
        dM/ddt y = -coll faci E.  ivis 2: the same on the off-diagonal
        stresses; on the diagonal ones M = faci (I + c J), c = coll dt/3, and
        since sum_d y_d = sum_d E_d there, (dM/ddt y)_d = -coll faci E_d +
        faci (coll/3) sum_k E_k."""
        g = (e - x) / dt
        iv = self.cfg.ivis
        if iv in (1, 2):
            faci = 1.0 / (1.0 + dt * coll)
            es, xs = e[:, PXX:], x[:, PXX:]
            g[:, PXX:] = (es - faci * xs) / dt - coll * faci * es
            if iv == 2:
                ed, xd = e[:, PXX:PZZ + 1], x[:, PXX:PZZ + 1]
                c3 = coll * dt / 3.0
                esum = ed.sum(1, keepdim=True)
                g[:, PXX:PZZ + 1] = ((ed - faci * (xd + c3 * xd.sum(1, keepdim=True))) / dt
                                     - coll * faci * ed + faci * (coll / 3.0) * esum)
        return (lam * g).sum()

    def _dcoll_stage(self, e, lam, dt: float, coll: float):
        """lam . dE/dcoll for the stage e = E(x) of ivis 1 (the stresses are
        faci (x - dt R) with faci = 1/(1 + dt coll) and R does not depend on
        coll, so dE/dcoll = -dt faci E there), a 0-d device tensor."""
        faci = 1.0 / (1.0 + dt * coll)
        return (lam[:, PXX:] * e[:, PXX:]).sum() * (-dt * faci)

    # ---- backward -----------------------------------------------------------
    def step_vjp(self, S: Solver, recs, lam, dt: float, coll: float, with_dt: bool = True,
                 with_dcoll: bool = True, n: int = 0):
        """Transpose of one step: (lam_q, dL/dcoll as a 0-d device tensor) from
        lam of its output.  For ivis 1 nothing in it waits for the device; for
        ivis 0 and 2, where coll enters the right-hand side, the stage VJPs
        return lam_out . dE/dcoll to the host (one synchronisation per stage)
        unless with_dcoll is False."""
        torch = _torch()
        iv = self.cfg.ivis
        torch_dc = with_dcoll and iv == 1
        kern_dc = with_dcoll and iv != 1
        acc = {"dcoll": torch.zeros((), dtype=lam.dtype, device=lam.device)}
        ddt = torch.zeros((), dtype=lam.dtype, device=lam.device)

        self._noise(S, n)

        def svjp(x, lam_out, e, k):
            self._noise(S, None, k)
            if kern_dc:
                out, dc = S.stage_vjp(x, lam_out, dt, e_out=e, want_dcoll=True)
                acc["dcoll"] = acc["dcoll"] + dc
                return out
            return S.stage_vjp(x, lam_out, dt)[0]

        def lvjp(xr, lam_x):   # through the limiter applied to xr, in place on lam_x
            return S.limiter_vjp(xr, lam_x, out=lam_x)

        if self.cfg.iorder == 2:
            (x0r, x0, e1), (x1r, x1, e2) = recs
            lam_e2 = 0.5 * lam
            lam_e1 = lvjp(x1r, svjp(x1, lam_e2, e2, 1))
            if torch_dc:
                acc["dcoll"] = acc["dcoll"] + self._dcoll_stage(e2, lam_e2, dt, coll) + self._dcoll_stage(e1, lam_e1, dt, coll)
            if with_dt:
                ddt = ddt + self._ddt_stage(x1, e2, lam_e2, dt, coll) + self._ddt_stage(x0, e1, lam_e1, dt, coll)
            lam_x0 = svjp(x0, lam_e1, e1, 0)
            lam_x0 += 0.5 * lam
        else:
            (x0r, x0, e1), (x1r, x1, e2), (x2r, x2, e3) = recs
            lam_e3 = (2.0 / 3.0) * lam
            lam_x2r = lvjp(x2r, svjp(x2, lam_e3, e3, 2))
            lam_e2 = 0.25 * lam_x2r
            lam_e1 = lvjp(x1r, svjp(x1, lam_e2, e2, 1))
            if torch_dc:
                acc["dcoll"] = (acc["dcoll"] + self._dcoll_stage(e3, lam_e3, dt, coll)
                                + self._dcoll_stage(e2, lam_e2, dt, coll) + self._dcoll_stage(e1, lam_e1, dt, coll))
            if with_dt:
                ddt = (ddt + self._ddt_stage(x2, e3, lam_e3, dt, coll) + self._ddt_stage(x1, e2, lam_e2, dt, coll)
                       + self._ddt_stage(x0, e1, lam_e1, dt, coll))
            lam_x0 = svjp(x0, lam_e1, e1, 0)
            lam_x0 += (1.0 / 3.0) * lam + 0.75 * lam_x2r
        lam_q = lvjp(x0r, lam_x0)
        if with_dt:
            lam_q += ddt * self._dt_grad(x0r, dt)
        return lam_q, acc["dcoll"]

    def backward(self, coll: float, ckpts, dts, lam, with_dt: bool = True, with_dcoll: bool = True):
        """(lam_q0, dL/dcoll) from lam of the final state (dL/dcoll 0.0 when
        with_dcoll is False)."""
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
                q, recs = self.step(S, q, dts[n], check=False, n=n)
                seg.append(recs)
            for n in range(end - 1, start - 1, -1):
                lam, dc = self.step_vjp(S, seg[n - start], lam, dts[n], coll, with_dt, with_dcoll, n)
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
            lam0, dcoll = ctx.roll.backward(ctx.coll, ctx.ckpts, ctx.dts, lam,
                                            with_dcoll=bool(ctx.needs_input_grad[1]))
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

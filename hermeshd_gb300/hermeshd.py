"""The reference's Python call surface (src/hermeshd.py:5-120), over the GB300 path.

Usage mirrors src/test_hermeshd.py:37-83::

    from hermeshd_gb300 import hermeshd, config
    hermeshd.hermeshd.configure(config.sod_1d())       # the reference: compile time
    setup, step = hermeshd.hermeshd.setup, hermeshd.hermeshd.step
    Qio = np.empty((nx, ny, nz, nQ, nB), order='F', dtype=np.float64)
    Q1, Q2 = np.empty_like(Qio), np.empty_like(Qio)
    t, dt = np.array(0.0), np.array(0.0)
    ...
    setup(Qio, t, dt, t1, t_start, dtout, nout, comm)
    while t < tf:
        step(Qio, Q1, Q2, t, dt)
        generate_output(Qio, t, dt, t1, dtout, nout)
    cleanup(t_start)

Arrays may be numpy Fortran-ordered host arrays (copied to the device and
back around each call, as the f2py extension works on host memory) or torch
CUDA tensors of shape (nbasis, nQ, nz, ny, nx) (no copies).  As with the
f2py extension's intent(inout) arguments, nothing is converted: a host array
must be Fortran-contiguous with the configuration's shape (nx, ny, nz, nQ,
nbasis) and its element type (float64 for precision 'fp64', float32 for
'fp32' -- the reference driver's float32 arrays, src/test_hermeshd.py:48-50,
run on the FP32 path); anything else raises HermesError with
HERMES_ERR_SHAPE or HERMES_ERR_DTYPE before any work is done.  Scalars are
0-d numpy arrays mutated in place, as in the reference, and are also
returned.  ``comm`` is accepted and ignored (one GPU, no MPI).
"""
from __future__ import annotations

import time
from typing import Optional

import numpy as np

from . import checkpoint as _ckpt
from . import ic as _ic
from . import output as _out
from ._lib import HermesError
from .config import Config
from .solver import Solver

_ERR_SHAPE, _ERR_DTYPE = 2, 3   # HERMES_ERR_SHAPE, HERMES_ERR_DTYPE (include/hermes_gb300.h)


def _set0d(a, v):
    if isinstance(a, np.ndarray) and a.ndim == 0:
        a[...] = v
    return v


def _get0d(a):
    return float(a) if a is not None else 0.0


class Hermeshd:
    """Module hermeshd (src/hermeshd.f90:2-269)."""

    def __init__(self):
        self.cfg: Optional[Config] = None
        self.icid: int = 3
        self.solver: Optional[Solver] = None
        self._dev = None
        # checkpoint switches of input.f90:99-103
        self.iwrite, self.iread, self.resuming, self.fpre, self.datadir = 0, 0, False, "Qout", "data"
        self.vtk, self.outdir, self.nvtk = False, "data", 1

    # ---- configuration (compile-time constants in the reference) --------
    def configure(self, cfg: Config, icid: Optional[int] = None, iwrite: int = 0, iread: int = 0,
                  resuming: bool = False, fpre: str = "Qout", datadir: str = "data", vtk: bool = False,
                  outdir: str = "data", nvtk: int = 1):
        """Select the problem: src/input.f90 and src/params.f90 at run time.
        icid follows initialcon.f90:41-69 (0 jet, 1/2 isentropic vortex
        v0/v1, 3/4 Sod v0/v1, 5-7 fluid at rest), built on the device; other
        problems set their own initial state.
        iwrite = 1 writes a checkpoint at every output (odd/even dump ids);
        iread = 1 or 2 starts from that dump, keeping its clock if resuming
        (input.f90:99-103).  vtk = True writes the VTK derived fields of
        output_vtk at every output into outdir (nvtk sub-cells per axis)."""
        cfg.validate()
        self.cfg = cfg
        if icid is not None:
            self.icid = icid
        self.iwrite, self.iread, self.resuming, self.fpre, self.datadir = iwrite, iread, resuming, fpre, datadir
        self.vtk, self.outdir, self.nvtk = vtk, outdir, nvtk
        if self.solver is not None:
            self.solver.close()
            self.solver = None

    def _check(self, a, name):
        """The f2py contract of an intent(inout) field array: a host array is
        used as given or rejected, never converted.  Device tensors are
        checked by the Solver (dtype, shape, contiguity, device)."""
        if a is None or not isinstance(a, np.ndarray):
            return
        cfg = self.cfg
        want = self._host_dtype()
        if a.dtype != want:
            raise HermesError(_ERR_DTYPE, f"{name}: dtype {a.dtype} does not match precision {cfg.precision} "
                                          f"(expected {np.dtype(want).name})")
        if tuple(a.shape) != tuple(cfg.shape_f):
            raise HermesError(_ERR_SHAPE, f"{name}: shape {tuple(a.shape)}, expected {tuple(cfg.shape_f)}")
        if not a.flags.f_contiguous:
            raise HermesError(_ERR_SHAPE, f"{name}: not Fortran-contiguous")

    def _host_dtype(self):
        return np.float64 if self.cfg.precision == "fp64" else np.float32

    def _need(self):
        if self.cfg is None:
            raise RuntimeError("hermeshd: configure(cfg) before setup (the reference fixes it at compile time)")
        if self.solver is None:
            self.solver = Solver(self.cfg)
        return self.solver

    # ---- the wrapped subprograms (CMakeLists.txt:161) ---------------------
    def main(self, comm=0):
        """hermeshd.f90:26-48: setup; while t < tf: step, generate_output; cleanup."""
        cfg = self.cfg
        Q = np.zeros(cfg.shape_f, order="F", dtype=self._host_dtype())
        Q1, Q2 = np.zeros_like(Q), np.zeros_like(Q)
        t, dt, t1, t_start, dtout, nout = (np.array(0.0), np.array(0.0), np.array(0.0), np.array(0.0),
                                            np.array(0.0), np.array(0))
        self.setup(Q, t, dt, t1, t_start, dtout, nout, comm)
        while float(t) < cfg.tf:
            self.step(Q, Q1, Q2, t, dt)
            self.generate_output(Q, t, dt, t1, dtout, nout)
        self.cleanup(t_start)
        return Q

    def setup(self, q_io, t, dt, t1, t_start, dtout, nout, comm=0):
        """hermeshd.f90:67-114: initializer (tables, spacing, dt), initial
        condition into q_io, integrator and boundary selection.  As set_ic
        does (initialcon.f90:29-32), ivis 0 zeroes coll and colvis."""
        if self.cfg is not None:
            self._check(q_io, "q_io")
        if self.cfg is not None and not self.iread and self.cfg.ivis == 0 and (self.cfg.coll or self.cfg.colvis):
            self.cfg = self.cfg.replace(coll=0.0, colvis=0.0)
            if self.solver is not None:
                self.solver.close()
                self.solver = None
        s = self._need()
        cfg = self.cfg
        _set0d(t, 0.0)
        _set0d(dt, cfg.cflm_eff * (cfg.lx / cfg.nx) / 2.0)      # initialize.f90:343 with clt = 2
        _set0d(nout, 0)
        now = time.time()
        _set0d(t_start, now)
        _set0d(dtout, cfg.tf / cfg.ntout)                      # hermeshd.f90:84
        if self.iread:
            # initialize.f90:396-438 set_ic_from_file
            Q, tr, dtr, nr = _ckpt.restart(self.datadir, cfg, self.iread, _get0d(dtout), self.resuming, self.fpre)
            if self.resuming:
                _set0d(t, tr)
                _set0d(dt, dtr)
                _set0d(nout, nr)
        elif 0 <= self.icid <= 7:
            # set_ic (initialcon.f90:20-72) built on the device
            dq = q_io if not isinstance(q_io, np.ndarray) else s.new_state()
            s.init_state(dq, self.icid)
            Q = s.to_numpy(dq) if isinstance(q_io, np.ndarray) else None
        else:
            Q = _ic.equilibrium(cfg)
        if Q is not None:
            self._write(q_io, Q)
        _set0d(t1, time.time())
        s.set_time(_get0d(t))
        return t, dt

    def _write(self, dst, Qf):
        if isinstance(dst, np.ndarray):
            dst[...] = Qf.astype(dst.dtype)
        else:
            dst.copy_(self.solver.from_numpy(Qf))

    def step(self, q_io, q_1, q_2, t, dt):
        """hermeshd.f90:53-62: dt = get_min_dt(Q); update(Q, Q1, Q2, dt); t += dt."""
        if self.cfg is not None:
            for a, name in ((q_io, "q_io"), (q_1, "q_1"), (q_2, "q_2")):
                self._check(a, name)
        s = self._need()
        if isinstance(q_io, np.ndarray):
            # host arrays: copy in, step, copy back (Q_1 returned as well),
            # in the arrays' own element type
            dq, d1 = s.from_numpy(q_io), s.from_numpy(q_1)
            tn, dtn = s.step(dq, d1, None, _get0d(t))
            q_io[...] = dq.cpu().numpy().T
            q_1[...] = d1.cpu().numpy().T
        else:
            tn, dtn = s.step(q_io, q_1, q_2, _get0d(t))
        _set0d(t, tn)
        _set0d(dt, dtn)
        return tn, dtn

    def generate_output(self, q_r, t, dt, t1, dtout, nout):
        """hermeshd.f90:206-266: when t passes the next output time, advance
        nout, write the VTK derived fields (output_vtk) when vtk is set and,
        with iwrite, the checkpoint with the odd/even dump id
        (hermeshd.f90:248-252)."""
        if self.cfg is not None:
            self._check(q_r, "q_r")
        if _get0d(t) > _get0d(nout) * _get0d(dtout):
            n = int(_get0d(nout)) + 1
            _set0d(nout, n)
            if self.vtk:
                s = self._need()
                q = s.from_numpy(q_r) if isinstance(q_r, np.ndarray) else q_r
                _out.output_vtk(s, q, n, outdir=self.outdir, nvtk=self.nvtk)
            if self.iwrite == 1:
                _ckpt.write_dump(self.datadir, q_r, _get0d(t), _get0d(dt), n, prefix=self.fpre)
        return nout

    def cleanup(self, t_start):
        """hermeshd.f90:119-138: release resources, report wall time."""
        wall = time.time() - _get0d(t_start)
        if self.solver is not None:
            self.solver.close()
            self.solver = None
        return wall


hermeshd = Hermeshd()

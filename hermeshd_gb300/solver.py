"""Device-side API over the C ABI: one DG problem (Solver) or an ensemble of
independent grids (Ensemble) advanced on the current torch CUDA stream.

Field arrays are torch tensors of shape (nbasis, nQ, nz, ny, nx), C-contiguous
-- the same memory as the reference's Fortran Q(nx,ny,nz,nQ,nbasis) -- with
dtype float64 (precision 'fp64') or float32 ('fp32').  torch provides device
memory and the stream; all arithmetic runs in the library's CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import check, lib, to_c
from .config import NQ, Config


def _torch():
    import torch
    return torch


class Solver:
    def __init__(self, cfg: Config, stream=None):
        torch = _torch()
        cfg.validate()
        self.cfg = cfg
        self.dtype = torch.float64 if cfg.precision == "fp64" else torch.float32
        self.np_dtype = np.float64 if cfg.precision == "fp64" else np.float32
        self.device = torch.device("cuda", torch.cuda.current_device())
        self.stream = stream if stream is not None else torch.cuda.current_stream(self.device)
        self._ccfg = to_c(cfg)
        self.ctx = C.c_void_p()
        self._create()
        self.nbox = 1

    def _create(self):
        check(lib().hermes_create(C.byref(self._ccfg), C.c_void_p(self.stream.cuda_stream), C.byref(self.ctx)))

    # ---- arrays ---------------------------------------------------------
    @property
    def shape(self):
        return self.cfg.shape_c

    def new_state(self):
        torch = _torch()
        return torch.zeros(self.shape, dtype=self.dtype, device=self.device)

    def from_numpy(self, Qf: np.ndarray):
        """Fortran-ordered Q(nx,ny,nz,nQ,nb) -> device tensor (nb,nQ,nz,ny,nx)."""
        torch = _torch()
        a = np.ascontiguousarray(np.asarray(Qf).T, dtype=self.np_dtype)
        return torch.from_numpy(a).to(self.device)

    def to_numpy(self, q) -> np.ndarray:
        """Device tensor -> Fortran-ordered float64 numpy array Q(nx,ny,nz,nQ,nb)."""
        return np.asfortranarray(q.detach().double().cpu().numpy().T)

    def _ptr(self, t):
        torch = _torch()
        if not isinstance(t, torch.Tensor):
            raise TypeError("expected a torch CUDA tensor")
        if t.dtype != self.dtype:
            raise _lib.HermesError(3, f"dtype {t.dtype} does not match precision {self.cfg.precision}")
        if tuple(t.shape) != tuple(self.shape) or not t.is_contiguous():
            raise _lib.HermesError(2, f"expected contiguous shape {self.shape}, got {tuple(t.shape)}")
        if t.device != self.device:
            raise _lib.HermesError(8, f"tensor on {t.device}, context on {self.device}")
        return C.c_void_p(t.data_ptr())

    # ---- operations -----------------------------------------------------
    def get_min_dt(self, q) -> float:
        dt = C.c_double()
        check(lib().hermes_get_min_dt(self.ctx, self._ptr(q), C.byref(dt)), self.ctx)
        return dt.value

    def limiter(self, q):
        check(lib().hermes_limiter(self.ctx, self._ptr(q)), self.ctx)
        return q

    def rhs(self, q, limit: bool = True, out=None):
        """glflux - source of q (q limited in place first when limit)."""
        out = self.new_state() if out is None else out
        check(lib().hermes_rhs(self.ctx, self._ptr(q), self._ptr(out), int(limit)), self.ctx)
        return out

    def euler_stage(self, q_in, dt: float, out=None):
        out = self.new_state() if out is None else out
        check(lib().hermes_euler_stage(self.ctx, self._ptr(q_in), self._ptr(out), float(dt)), self.ctx)
        return out

    # ---- adjoint (FP64, one grid) -------------------------------------------
    def rhs_vjp(self, q, mu, out=None):
        """(dR/dq)^T mu for R = rhs(q, limit=False)."""
        out = self.new_state() if out is None else out
        check(lib().hermes_rhs_vjp(self.ctx, self._ptr(q), self._ptr(mu), self._ptr(out)), self.ctx)
        return out

    def limiter_vjp(self, q, lam_out, out=None):
        """(dL/dq)^T lam_out for the positivity limiter L applied in place at
        q (the stage input before limiting): the derivative of the branch it
        takes there.  out may be lam_out."""
        out = self.new_state() if out is None else out
        check(lib().hermes_limiter_vjp(self.ctx, self._ptr(q), self._ptr(lam_out), self._ptr(out)), self.ctx)
        return out

    def stage_vjp(self, q_in, lam_out, dt: float, e_out=None, want_dcoll: bool = False, out=None):
        """(dE/dq_in)^T lam_out for the forward-Euler stage E of
        euler_stage(q_in, dt) (limiter inactive); with want_dcoll also
        lam_out . dE/dcoll (needs e_out = E(q_in); synchronises).  Returns
        (lam_in, dcoll or None)."""
        out = self.new_state() if out is None else out
        dc = C.c_double(0.0)
        check(lib().hermes_stage_vjp(self.ctx, self._ptr(q_in), None if e_out is None else self._ptr(e_out),
                                     self._ptr(lam_out), self._ptr(out), float(dt),
                                     C.byref(dc) if want_dcoll else None), self.ctx)
        return out, (dc.value if want_dcoll else None)

    def step(self, q, q1, q2=None, t: float = 0.0):
        """One step of hermeshd.f90:53-62; returns (t, dt)."""
        tt, dd = C.c_double(t), C.c_double(0.0)
        check(lib().hermes_step(self.ctx, self._ptr(q), self._ptr(q1), None if q2 is None else self._ptr(q2),
                                C.byref(tt), C.byref(dd)), self.ctx)
        return tt.value, dd.value

    def advance(self, q, q1, nsteps: int, t: float = 0.0):
        """nsteps steps from one captured CUDA graph; returns (t, dt)."""
        tt, dd = C.c_double(t), C.c_double(0.0)
        check(lib().hermes_advance(self.ctx, self._ptr(q), self._ptr(q1), None, int(nsteps), C.byref(tt),
                                   C.byref(dd)), self.ctx)
        return tt.value, dd.value

    def enqueue_steps(self, q, q1, nsteps: int):
        """nsteps steps enqueued on the context stream, no synchronisation."""
        check(lib().hermes_enqueue_steps(self.ctx, self._ptr(q), self._ptr(q1), int(nsteps)), self.ctx)

    @property
    def cuda_stream(self) -> int:
        """The private stream the kernels run on (cudaStream_t as int)."""
        return int(lib().hermes_stream(self.ctx) or 0)

    def profile(self, enable: bool = True):
        check(lib().hermes_profile_enable(self.ctx, int(enable)), self.ctx)

    KERNEL_KINDS = ("cfl_dt", "limiter", "face_x", "face_y", "face_z", "cell", "noise", "trace", "tile")

    def profile_read(self):
        ms = np.zeros(len(self.KERNEL_KINDS))
        n = np.zeros(len(self.KERNEL_KINDS), dtype=np.int64)
        check(lib().hermes_profile_read(self.ctx, ms.ctypes.data_as(C.POINTER(C.c_double)),
                                        n.ctypes.data_as(C.POINTER(C.c_int64))), self.ctx)
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(self.KERNEL_KINDS)}

    def advance_host(self, q_host: np.ndarray, nsteps: int, t: float = 0.0):
        """nsteps on a host array (C-contiguous (nb,nQ,nz,ny,nx) or Fortran
        Q(nx,ny,nz,nQ,nb), dtype matching the precision), updated in place."""
        if q_host.dtype != self.np_dtype:
            raise _lib.HermesError(3, "host array dtype does not match the precision")
        # the two views of the same memory; a C-ordered Q(nx,ny,nz,nQ,nb) has the
        # right size but another layout, and is refused rather than misread
        sh = tuple(self.shape)
        if not ((q_host.shape == sh and q_host.flags.c_contiguous) or
                (q_host.shape == sh[::-1] and q_host.flags.f_contiguous)):
            raise _lib.HermesError(2, f"expected a C-contiguous {sh} or Fortran-ordered {sh[::-1]} host array, "
                                      f"got shape {q_host.shape} (C-contiguous {q_host.flags.c_contiguous}, "
                                      f"Fortran {q_host.flags.f_contiguous})")
        tt, dd = C.c_double(t), C.c_double(0.0)
        check(lib().hermes_advance_host(self.ctx, C.c_void_p(q_host.ctypes.data), int(nsteps), C.byref(tt),
                                        C.byref(dd)), self.ctx)
        return tt.value, dd.value

    def init_state(self, q, icid: int, seed: int = 0):
        """Fill q on the device with the initial state of set_ic problem icid
        (0 jet, 1/2 vortex v0/v1, 3/4 Sod v0/v1, 5-7 fluid at rest)."""
        check(lib().hermes_init_state(self.ctx, self._ptr(q), int(icid), int(seed)), self.ctx)
        return q

    def conserved(self, q) -> np.ndarray:
        """FP64 integrals of rho, m_x, m_y, m_z, E per box: array (nbox, 5)."""
        out = np.zeros((self.nbox, 5))
        check(lib().hermes_conserved(self.ctx, self._ptr(q), out.ctypes.data_as(C.POINTER(C.c_double))), self.ctx)
        return out

    # ---- launch shape ---------------------------------------------------------
    def get_launch(self) -> dict:
        l = _lib.HermesLaunch()
        check(lib().hermes_get_launch(self.ctx, C.byref(l)), self.ctx)
        return {"face_tpb": l.face_tpb, "dt_tpb": l.dt_tpb, "steps_per_graph": l.steps_per_graph,
                "noise_inline": l.noise_inline, "face_traces": l.face_traces, "split_update": l.split_update,
                "tile_stage": l.tile_stage, "pdl": l.pdl,
                "faces_merged": l.faces_merged, "update_tpb": l.update_tpb, "cell_concurrent": l.cell_concurrent}

    def set_launch(self, face_tpb: int = 0, dt_tpb: int = 0, steps_per_graph: int = 1, noise_inline: int = 0,
                   face_traces=None, split_update=None, tile_stage=None, pdl=None,
                   faces_merged=None, update_tpb: int = 0, cell_concurrent=None):
        """face_traces / split_update / tile_stage None keep the context's
        current choice (the trace kernel and the split update are on by
        default where they exist: FP64 nbasis 8/10 without the stochastic
        stress, and ivis 0/1; the fused stage, nbasis 4 ivis 0/1, is off by
        default); pdl None keeps the current choice (off by default); faces_merged None keeps
        the current choice (1: one launch for three directions, the default in
        FP64; 0: one per direction, nbasis 8/10 in FP32 and nbasis 4 in FP32
        below 2^15 cells; 2: one per direction with a thread per face looping
        over its points, nbasis 4 in FP32 from 2^15 cells);
        update_tpb: threads per block of the split update (0: the default,
        64 in FP32, 128 in FP64); cell_concurrent None keeps the current choice
        (1, the default: the split update's volume kernel on a second stream
        beside the trace and face kernels; 0: one stream)."""
        cur = self.get_launch()
        if face_traces is None:
            face_traces = cur["face_traces"]
        if split_update is None:
            split_update = cur["split_update"]
        if tile_stage is None:
            tile_stage = cur["tile_stage"]
        if pdl is None:
            pdl = cur["pdl"]
        if faces_merged is None:
            faces_merged = cur["faces_merged"]
        if cell_concurrent is None:
            cell_concurrent = cur["cell_concurrent"]
        l = _lib.HermesLaunch(int(face_tpb), int(dt_tpb), int(steps_per_graph), int(noise_inline), int(face_traces),
                              int(split_update), int(tile_stage), int(pdl), int(faces_merged), int(update_tpb),
                              int(cell_concurrent))
        check(lib().hermes_set_launch(self.ctx, C.byref(l)), self.ctx)

    def set_noise_step(self, step: int):
        check(lib().hermes_set_noise_step(self.ctx, int(step)), self.ctx)

    def set_noise_stage(self, stage: int):
        """Stage index (0..2) of the stochastic-stress draw of rhs,
        euler_stage and the VJPs (step and advance count their own stages)."""
        check(lib().hermes_set_noise_stage(self.ctx, int(stage)), self.ctx)

    def set_time(self, t: float):
        check(lib().hermes_set_time(self.ctx, float(t)), self.ctx)

    def check(self):
        check(lib().hermes_check(self.ctx), self.ctx)

    def close(self):
        if getattr(self, "ctx", None) and self.ctx.value:
            lib().hermes_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ensemble(Solver):
    """nbox independent grids of one physics configuration, stored back to
    back in one flat tensor; each box has its own CFL time step, time and
    Philox key."""

    def __init__(self, cfg: Config, dims: Sequence[Sequence[int]], lengths: Optional[Sequence[Sequence[float]]] = None,
                 seeds: Optional[Sequence[int]] = None, stream=None):
        self._dims = np.ascontiguousarray(np.asarray(dims, dtype=np.int32).reshape(-1, 3))
        self._lengths = None if lengths is None else np.ascontiguousarray(np.asarray(lengths, dtype=np.float64).reshape(-1, 3))
        self._seeds = None if seeds is None else np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64))
        super().__init__(cfg, stream)
        self.nbox = len(self._dims)
        off = np.zeros(self.nbox + 1, dtype=np.int64)
        check(lib().hermes_box_offsets(self.ctx, off.ctypes.data_as(C.POINTER(C.c_int64))), self.ctx)
        self.offsets = off

    def _create(self):
        n = len(self._dims)
        dims = self._dims.ctypes.data_as(C.POINTER(C.c_int32))
        lens = None if self._lengths is None else self._lengths.ctypes.data_as(C.POINTER(C.c_double))
        seeds = None if self._seeds is None else self._seeds.ctypes.data_as(C.POINTER(C.c_uint64))
        check(lib().hermes_ensemble_create(C.byref(self._ccfg), n, dims, lens, seeds,
                                           C.c_void_p(self.stream.cuda_stream), C.byref(self.ctx)))

    @property
    def shape(self):
        return (int(self.offsets[-1]),) if hasattr(self, "offsets") else None

    @property
    def ncells(self):
        return int(np.prod(self._dims, axis=1).sum())

    @property
    def dof(self):
        return self.ncells * NQ * self.cfg.nbasis

    def box_view(self, q, i):
        """(nb, nQ, nz, ny, nx) view of box i of a flat ensemble tensor."""
        nx, ny, nz = (int(v) for v in self._dims[i])
        return q[int(self.offsets[i]):int(self.offsets[i + 1])].view(self.cfg.nbasis, NQ, nz, ny, nx)

    def box_times(self):
        t = np.zeros(self.nbox)
        dt = np.zeros(self.nbox)
        check(lib().hermes_box_times(self.ctx, t.ctypes.data_as(C.POINTER(C.c_double)),
                                     dt.ctypes.data_as(C.POINTER(C.c_double))), self.ctx)
        return t, dt

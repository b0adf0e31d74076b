"""Checkpoint files of the reference's writeQ / readQ (initialize.f90:474-565)
with its odd/even rotation (hermeshd.f90:248-252) and restart checks
(initialize.f90:396-438), over the library's C text reader/writer.

A checkpoint is data/<prefix>_p<rank:04d>_d<dump:04d>.dat: one record per
(basis, variable, k, j) with the nx values of the row, then
"t dt nout mpi_nx mpi_ny mpi_nz".  Fields are FP64 Q(nx,ny,nz,nQ,nbasis) host
arrays in Fortran order, or the library's device tensors (copied through a
pinned host buffer).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence, Tuple

import numpy as np

from . import _lib
from .config import Config


def checkpoint_name(prefix: str = "Qout", rank: int = 0, dump: int = 1) -> str:
    """writeQ's file name (initialize.f90:484-497): 4-digit rank and dump id."""
    return f"{prefix}_p{rank:04d}_d{dump:04d}.dat"


def odd_even_dump(nout: int) -> int:
    """hermeshd.f90:249: dump id 1 or 2, so the last two checkpoints are kept."""
    return 2 - nout % 2


def _host_f64(q) -> np.ndarray:
    """Fortran-ordered FP64 host copy of a device tensor (nb,nQ,nz,ny,nx) or a host array."""
    if isinstance(q, np.ndarray):
        a = np.asarray(q, dtype=np.float64)
        return a if a.flags.f_contiguous else np.asfortranarray(a)
    import torch
    h = torch.empty(q.shape, dtype=torch.float64, pin_memory=True)
    h.copy_(q.detach())
    return h.numpy().T      # C-contiguous (nb,nQ,nz,ny,nx) viewed as Fortran (nx,ny,nz,nQ,nb)


def write(path: str, q, t: float, dt: float, nout: int, mpi_dims: Sequence[int] = (1, 1, 1)) -> str:
    a = _host_f64(q)
    nx, ny, nz, nq, nb = a.shape
    err = C.create_string_buffer(256)
    md = (C.c_int32 * 3)(*[int(x) for x in mpi_dims])
    rc = _lib.lib().hermes_checkpoint_write(os.fsencode(path), C.c_void_p(a.ctypes.data), nx, ny, nz, nb,
                                            float(t), float(dt), int(nout), md, err, 256)
    if rc:
        raise _lib.HermesError(rc, err.value.decode())
    return path


def read(path: str, cfg: Config) -> Tuple[np.ndarray, float, float, int, Tuple[int, int, int]]:
    """(Q, t, dt, nout, mpi_dims) of a checkpoint for cfg's grid."""
    Q = np.zeros(cfg.shape_f, dtype=np.float64, order="F")
    t, dt = C.c_double(0.0), C.c_double(0.0)
    nout = C.c_int32(0)
    md = (C.c_int32 * 3)(1, 1, 1)
    err = C.create_string_buffer(256)
    rc = _lib.lib().hermes_checkpoint_read(os.fsencode(path), C.c_void_p(Q.ctypes.data), cfg.nx, cfg.ny, cfg.nz,
                                           cfg.nbasis, C.byref(t), C.byref(dt), C.byref(nout), md, err, 256)
    if rc:
        raise _lib.HermesError(rc, err.value.decode())
    return Q, t.value, dt.value, nout.value, (md[0], md[1], md[2])


def write_dump(directory: str, q, t: float, dt: float, nout: int, prefix: str = "Qout", rank: int = 0,
               dump: Optional[int] = None, mpi_dims: Sequence[int] = (1, 1, 1)) -> str:
    """writeQ into directory with the odd/even dump id of nout unless dump is given."""
    os.makedirs(directory, exist_ok=True)
    d = odd_even_dump(nout) if dump is None else dump
    return write(os.path.join(directory, checkpoint_name(prefix, rank, d)), q, t, dt, nout, mpi_dims)


def restart(directory: str, cfg: Config, dump: int, dtout: float, resuming: bool, prefix: str = "Qout",
            rank: int = 0, mpi_dims: Sequence[int] = (1, 1, 1)):
    """set_ic_from_file (initialize.f90:396-438): read the dump; when resuming
    keep its t, dt and nout, else start at t = 0, nout = 0.  The reference's
    consistency checks raise instead of exiting: dtout must match the file's
    t/(nout-1) within 1.01 of its dt, and the MPI layout must match.
    Returns (Q, t, dt, nout)."""
    Q, t_p, dt_p, nout_p, md = read(os.path.join(directory, checkpoint_name(prefix, rank, dump)), cfg)
    t, dt, nout = (t_p, dt_p, nout_p) if resuming else (0.0, 0.0, 0)
    dtout_p = t_p / (nout_p - 1) if nout > 1 else dtout
    if dt_p != 0.0 and abs(dtout_p - dtout) / dt_p > 1.01:
        raise _lib.HermesError(1, "bad restart, non-matching dtout")
    if tuple(md) != tuple(int(x) for x in mpi_dims):
        raise _lib.HermesError(1, "bad restart, non-matching mpi_nx, mpi_ny or mpi_nz")
    return Q, t, dt, nout

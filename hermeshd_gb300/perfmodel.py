"""Algorithmic cost model of one RK stage, for roofline reporting.

Bytes: a stage reads the stage input and writes the stage output once per
DOF (2s bytes, s = 8 for FP64, 4 for FP32); a stage that also folds in Q^n
(RK2 stage 2, RK3 stages 2 and 3) reads it too (3s).  Averaged per stage:
RK2 2.5s, RK3 8s/3.  The CFL reduction and the tables add nothing.

Flops: algorithmic floating-point operations of one cell and one stage, with
the basis/quadrature products counted only where the table entry is nonzero
(the kernels skip the zeros at compile time), a fused multiply-add counted
as 2, and a division or square root as 1.  The per-point physics counts are
read off dg_physics.cuh (point flux, primitives, HLLC).
"""
from __future__ import annotations

import os
import sys

from .config import NQ, Config

_CSRC = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc")

# per-point physics operation counts (dg_physics.cuh)
PRIM = 18            # primitives(): 1/rho, velocities, |m|^2, P, P_10
PFLUX = 28           # point_flux(), ivis 0/1, one direction
HLLC = 72            # hllc(): wave speeds (2 sqrt), S_M, p*, one star state, selection
CENTRAL = 2 * NQ     # 0.5*(fL + fR)
SCALE = NQ           # multiply by the inverse spacing
UPDATE = 5           # Q - dt*R, faci, RK combination, per (b, v)
DT_CELL = 20         # CFL reduction per cell


def _tables(nb, iq):
    if _CSRC not in sys.path:
        sys.path.insert(0, _CSRC)
    import gen_tables
    return gen_tables.tables(nb, iq)


def _nnz(row):
    return sum(1 for v in row if v != 0.0)


def bytes_per_dof_stage(precision: str, iorder: int) -> float:
    s = 8 if precision == "fp64" else 4
    return (2 * s + 3 * s) / 2 if iorder == 2 else (2 * s + 3 * s + 3 * s) / 3


def flops_per_cell_stage(cfg: Config) -> dict:
    T = _tables(cfg.nbasis, cfg.iquad)
    nf, npg = cfg.iquad ** 2, cfg.iquad ** 3
    # faces: 3 faces per cell (each face belongs to one cell in a periodic grid)
    face_pt = 0
    for d, (P, M) in enumerate((("XP", "XM"), ("YP", "YM"), ("ZP", "ZM"))):
        for p in range(nf):
            face_pt += 2 * NQ * (_nnz(T[P][p]) + _nnz(T[M][p]))
    face_pt += 3 * nf * (2 * PRIM + 2 * PFLUX + CENTRAL + SCALE + (HLLC if cfg.ihllc else 0))
    # cell: interior values, point fluxes, volume quadrature, surface, update
    interior = sum(2 * NQ * _nnz(T["INT"][g]) for g in range(npg))
    points = npg * (PRIM + 3 * (PFLUX + SCALE))
    volume = sum(2 * NQ * (_nnz(T["VX"][g]) + _nnz(T["VY"][g]) + _nnz(T["VZ"][g])) for g in range(npg))
    surface = sum(2 * NQ * _nnz(T[k][p]) for k in ("SXP", "SXM", "SYP", "SYM", "SZP", "SZM") for p in range(nf))
    source = 0
    if cfg.ivis == 0:
        source = npg * 6 + sum(2 * 6 * _nnz(T["SRC"][g]) for g in range(npg))
    update = UPDATE * NQ * cfg.nbasis
    limiter = 2 * 5 * (cfg.nbasis - 1) + 25        # the bound test (the point-wise path runs only near floors)
    parts = dict(face=face_pt, cell=interior + points + volume + surface + source + update, limiter=limiter,
                 cfl=DT_CELL / cfg.stages)
    parts["total"] = sum(parts.values())
    return parts


def flops_per_dof_stage(cfg: Config) -> float:
    return flops_per_cell_stage(cfg)["total"] / (NQ * cfg.nbasis)

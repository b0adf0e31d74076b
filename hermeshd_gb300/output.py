"""VTK output of the reference (output.f90:14-317): derived fields computed on
the device (hermes_derived) and written as a VTK XML rectilinear grid,
headless, one file per output: <outdir>/perseus_p<rank:04d>_t<nout:04d>.vtr.

Variables (index = bit of the selection mask), with the reference's VTK names:
"""
from __future__ import annotations

import base64
import ctypes as C
import os
import struct
from typing import Dict, Optional, Sequence

import numpy as np

from . import _lib
from .config import Config, Units

VARIABLES = ("Density", "Log density", "Velocity_x", "Velocity_y", "Velocity_z", "Temperature",
             "Internal energy density", "Total energy density", "Entropy density", "Pressure",
             "Isotropic stress_xx", "Isotropic stress_yy", "Isotropic stress_zz", "Vorticity")
# the reference's default selection (input.f90:87-96): density, velocity, temperature, pressure
DEFAULT = ("Density", "Velocity", "Temperature", "Pressure")
GROUPS = {"Velocity": ("Velocity_x", "Velocity_y", "Velocity_z"),
          "Isotropic stress": ("Isotropic stress_xx", "Isotropic stress_yy", "Isotropic stress_zz")}
__doc__ += "".join(f"\n  {i:2d} {n}" for i, n in enumerate(VARIABLES))


def _expand(names: Sequence[str]):
    out = []
    for n in names:
        out.extend(GROUPS.get(n, (n,)))
    for n in out:
        if n not in VARIABLES:
            raise KeyError(n)
    return out


def units_of(u: Optional[Units] = None) -> "_lib.HermesOutputUnits":
    """Output units of params.f90:80-94 (L0 = t0 = 1, v0 = L0/t0)."""
    u = u or Units()
    return _lib.HermesOutputUnits(u.n0, 1.0, 1.0, u.te0, u.eV_per_K)


def derived(solver, q, names: Sequence[str] = DEFAULT, nvtk: int = 1, units: Optional[Units] = None, out=None):
    """Selected variables as a float32 device tensor (nvar, nz*nvtk, ny*nvtk, nx*nvtk)
    in VARIABLES order, and the list of their names."""
    import torch
    sel = sorted(set(_expand(names)), key=VARIABLES.index)
    mask = sum(1 << VARIABLES.index(n) for n in sel)
    c = solver.cfg
    shape = (len(sel), c.nz * nvtk, c.ny * nvtk, c.nx * nvtk)
    if out is None:
        out = torch.empty(shape, dtype=torch.float32, device=solver.device)
    elif tuple(out.shape) != shape or out.dtype != torch.float32 or not out.is_contiguous():
        raise _lib.HermesError(2, f"out must be a contiguous float32 tensor of shape {shape}")
    u = units_of(units)
    _lib.check(_lib.lib().hermes_derived(solver.ctx, solver._ptr(q), C.c_void_p(out.data_ptr()), int(nvtk),
                                         int(mask), C.byref(u)), solver.ctx)
    return out, sel


def _data_array(name: str, a: np.ndarray, ncomp: int = 1) -> str:
    raw = np.ascontiguousarray(a, dtype="<f4").tobytes()
    b64 = base64.b64encode(struct.pack("<I", len(raw)) + raw).decode()
    return (f'        <DataArray type="Float32" Name="{name}" NumberOfComponents="{ncomp}" format="binary">\n'
            f"          {b64}\n        </DataArray>\n")


def write_vtr(path: str, cfg: Config, fields: Dict[str, np.ndarray], nvtk: int = 1) -> str:
    """VTK XML RectilinearGrid with cell data; fields: name -> (nz', ny', nx')
    array, or (3, nz', ny', nx') for a vector.  Sub-cell faces at
    xvtk - dxvtk/2 on the domain centred at the origin (params.f90:248-251)."""
    nnx, nny, nnz = cfg.nx * nvtk, cfg.ny * nvtk, cfg.nz * nvtk
    xs = [-cfg.lx / 2 + i * cfg.lx / nnx for i in range(nnx + 1)]
    ys = [-cfg.ly / 2 + j * cfg.ly / nny for j in range(nny + 1)]
    zs = [-cfg.lz / 2 + k * cfg.lz / nnz for k in range(nnz + 1)]
    ext = f"0 {nnx} 0 {nny} 0 {nnz}"
    parts = ['<?xml version="1.0"?>\n',
             '<VTKFile type="RectilinearGrid" version="0.1" byte_order="LittleEndian" header_type="UInt32">\n',
             f'  <RectilinearGrid WholeExtent="{ext}">\n', f'    <Piece Extent="{ext}">\n',
             "      <Coordinates>\n",
             _data_array("X", np.array(xs)), _data_array("Y", np.array(ys)), _data_array("Z", np.array(zs)),
             "      </Coordinates>\n", "      <CellData>\n"]
    for name, a in fields.items():
        a = np.asarray(a)
        if a.ndim == 4:   # vector: interleave components per cell
            parts.append(_data_array(name, np.stack([c.reshape(-1) for c in a], axis=1), 3))
        else:
            parts.append(_data_array(name, a.reshape(-1)))
    parts += ["      </CellData>\n", "    </Piece>\n", "  </RectilinearGrid>\n", "</VTKFile>\n"]
    with open(path, "w") as f:
        f.write("".join(parts))
    return path


def output_vtk(solver, q, nout: int, rank: int = 0, outdir: str = "data", names: Sequence[str] = DEFAULT,
               nvtk: int = 1, units: Optional[Units] = None) -> str:
    """output_vtk (output.f90:14-317): derived fields on the device, one .vtr file."""
    arr, sel = derived(solver, q, names, nvtk, units)
    host = arr.cpu().numpy()
    fields = {}
    for n in names:
        comps = GROUPS.get(n, (n,))
        idx = [sel.index(c) for c in comps]
        fields[n] = host[idx[0]] if len(idx) == 1 else host[idx]
    os.makedirs(outdir, exist_ok=True)
    return write_vtr(os.path.join(outdir, f"perseus_p{rank:04d}_t{nout:04d}.vtr"), solver.cfg, fields, nvtk)

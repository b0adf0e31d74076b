"""Ensemble statistics of fluctuating-hydro runs, on the device.

StructureFactor accumulates the static structure factor of the density,
S(k) = < |delta rho_hat(k)|^2 > / N_cells, from the cell averages of every box
of an ensemble (or of single grids), binned in shells of integer |k|
(wavenumbers in units of 2 pi / L of each box).  torch.fft does the
transforms; the grids are the library's field arrays.
"""
from __future__ import annotations

import math
from typing import Dict, Iterable, Optional

import numpy as np

from .config import NQ


class StructureFactor:
    def __init__(self, kmax: int = 32, var: int = 0):
        self.kmax = kmax
        self.var = var            # which conserved variable (0 = density)
        self.sum = np.zeros(kmax + 1)
        self.count = np.zeros(kmax + 1)
        self.samples = 0

    def add_grid(self, cell_avg):
        """cell_avg: torch tensor (nz, ny, nx) of one box's cell averages."""
        import torch
        a = cell_avg.double()
        d = a - a.mean()
        n = d.numel()
        F = torch.fft.fftn(d)
        P = (F.real ** 2 + F.imag ** 2) / n
        nz, ny, nx = d.shape
        kz = torch.fft.fftfreq(nz, d=1.0 / nz, device=d.device)
        ky = torch.fft.fftfreq(ny, d=1.0 / ny, device=d.device)
        kx = torch.fft.fftfreq(nx, d=1.0 / nx, device=d.device)
        K = torch.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2)
        shell = torch.round(K).long().clamp(max=self.kmax + 1)
        s = torch.zeros(self.kmax + 2, dtype=torch.float64, device=d.device).index_add_(0, shell.flatten(), P.flatten())
        c = torch.zeros(self.kmax + 2, dtype=torch.float64, device=d.device).index_add_(
            0, shell.flatten(), torch.ones_like(P).flatten())
        s, c = s[: self.kmax + 1].cpu().numpy(), c[: self.kmax + 1].cpu().numpy()
        # k = 0 holds the removed mean: exclude it
        s[0] = 0.0
        c[0] = 0.0
        self.sum += s
        self.count += c
        self.samples += 1

    def add_state(self, q, nb: int, dims=None, offsets=None):
        """Add every box of a field array: q is (nb, nQ, nz, ny, nx) for one
        grid, or the flat ensemble tensor with dims/offsets."""
        if dims is None:
            self.add_grid(q[0, self.var])
            return
        for i, (nx, ny, nz) in enumerate(dims):
            box = q[int(offsets[i]):int(offsets[i + 1])].view(nb, NQ, nz, ny, nx)
            self.add_grid(box[0, self.var])

    def result(self) -> Dict[int, float]:
        out = {}
        for k in range(1, self.kmax + 1):
            if self.count[k] > 0:
                out[k] = float(self.sum[k] / self.count[k])
        return out

    def flatness(self, kmin: int = 1, kmax: Optional[int] = None) -> float:
        """Relative spread (std/mean) of S(k) over the shells kmin..kmax."""
        r = self.result()
        ks = [k for k in r if k >= kmin and (kmax is None or k <= kmax)]
        v = np.array([r[k] for k in ks])
        return float(v.std() / v.mean()) if len(v) > 1 and v.mean() != 0 else math.nan

"""Derived fields of the reference's VTK output (output.f90:14-317), restated
in numpy (TEST INFRASTRUCTURE ONLY: only tests/ and bench.py's CPU legs use it).

bfvtk / bfvtk_dx / bfvtk_dy follow set_vtk_vals_3D (basis_funcs.f90:88-200)
term by term, with the basis index map of the oracle (set_basis_function_flags,
initialize.f90:126-194, via orc_get_kindex).  Variables in the order of
hermes_derived: 0 density*n0, 1 log10 density*n0, 2-4 velocity*v0,
5 temperature, 6 internal energy density, 7 total energy density, 8 entropy
density, 9 pressure, 10-12 pxx/pyy/pzz, 13 vorticity.
"""
import numpy as np

import oracle as O

RH, MX, MY, MZ, EN, PXX, PYY, PZZ = 0, 1, 2, 3, 4, 5, 6, 7


def vtk_tables(cfg, nvtk):
    """(bfvtk, bfvtk_dx, bfvtk_dy) of shape (nvtk^3, nbasis)."""
    o = O.Oracle(cfg)
    k = dict(zip(("kx", "ky", "kz", "kyz", "kzx", "kxy", "kxyz", "kxx", "kyy", "kzz", "kyzz", "kzxx", "kxyy",
                  "kyyz", "kzzx", "kxxy", "kyyzz", "kzzxx", "kxxyy", "kyzxx", "kzxyy", "kxyzz", "kxyyzz",
                  "kyzzxx", "kzxxyy", "kxxyyzz", "kxxx", "kyyy", "kzzz"), (int(v) - 1 for v in o.kindex())))
    nb = cfg.nbasis
    xgrid = {1: [0.0], 2: [-0.5, 0.5], 3: [-2.0 / 3.0, 0.0, 2.0 / 3.0], 4: [-0.75, -0.25, 0.25, 0.75]}[nvtk]
    n3 = nvtk ** 3
    W = max(k.values()) + 2
    bf = np.zeros((n3, W))
    bf[:, 0] = 1.0
    for i in range(nvtk):                                   # basis_funcs.f90:124-133
        bf[i * nvtk:(i + 1) * nvtk, k["ky"]] = xgrid[i]
        bf[i * nvtk:(i + 1) * nvtk, k["kz"]] = xgrid
    for i in range(nvtk):
        bf[i * nvtk * nvtk:(i + 1) * nvtk * nvtk, k["kx"]] = xgrid[i]
        bf[i * nvtk * nvtk:(i + 1) * nvtk * nvtk, k["ky"]] = bf[:nvtk * nvtk, k["ky"]]
        bf[i * nvtk * nvtk:(i + 1) * nvtk * nvtk, k["kz"]] = bf[:nvtk * nvtk, k["kz"]]
    x, y, z = bf[:, k["kx"]].copy(), bf[:, k["ky"]].copy(), bf[:, k["kz"]].copy()
    P2 = lambda s: 1.5 * s ** 2 - 0.5
    dx = np.zeros_like(bf)
    dy = np.zeros_like(bf)
    dx[:, k["kx"]] = 1.0
    dy[:, k["ky"]] = 1.0
    for name, val, vdx, vdy in (
            ("kyz", y * z, 0 * x, z), ("kzx", z * x, z, 0 * x), ("kxy", x * y, y, x), ("kxyz", x * y * z, y * z, z * x),
            ("kxx", P2(x), 3 * x, 0 * x), ("kyy", P2(y), 0 * x, 3 * y), ("kzz", P2(z), 0 * x, 0 * x)):
        if k[name] < nb:
            bf[:, k[name]] = val
            dx[:, k[name]] = vdx
            dy[:, k[name]] = vdy
    return bf[:, :nb], dx[:, :nb], dy[:, :nb]


def derived(cfg, Q, nvtk=1, n0=1.0, v0=1.0, t0=1.0, te0=1.0, eV_per_K=1.0):
    """(14, nnz, nny, nnx) float64 array of the variables of output_vtk."""
    bf, bdx, bdy = vtk_tables(cfg, nvtk)
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    out = np.zeros((14, nz * nvtk, ny * nvtk, nx * nvtk))
    g = cfg.aindex
    dxi = cfg.nx / cfg.lx
    for ib in range(nvtk):
        for jb in range(nvtk):
            for kb in range(nvtk):
                igrid = nvtk * nvtk * ib + nvtk * jb + kb          # output.f90:112
                q = np.einsum("b,ijkvb->ijkv", bf[igrid], Q[:, :, :, :8, :])
                dxrh = np.einsum("b,ijkb->ijk", bdx[igrid], Q[:, :, :, RH, :])
                dyrh = np.einsum("b,ijkb->ijk", bdy[igrid], Q[:, :, :, RH, :])
                dxmy = np.einsum("b,ijkb->ijk", bdx[igrid], Q[:, :, :, MY, :])
                dymx = np.einsum("b,ijkb->ijk", bdy[igrid], Q[:, :, :, MX, :])
                dn = q[..., RH]
                dni = 1.0 / dn
                vx, vy, vz = q[..., MX] * dni, q[..., MY] * dni, q[..., MZ] * dni
                U = q[..., EN] - 0.5 * dn * (vx ** 2 + vy ** 2 + vz ** 2)
                P = (g - 1.0) * U
                dxvy = (dn * dxmy - q[..., MY] * dxrh) / dn ** 2
                dyvx = (dn * dymx - q[..., MX] * dyrh) / dn ** 2
                vals = [dn * n0, np.log(dn * n0) / np.log(10.0), v0 * q[..., MX] / dn, v0 * q[..., MY] / dn,
                        v0 * q[..., MZ] / dn, P * te0 * dni / eV_per_K, U, q[..., EN], P * dni ** (g - 1.0), P,
                        q[..., PXX], q[..., PYY], q[..., PZZ], -2.0 * (dxvy - dyvx) * dxi / t0]
                for v, a in enumerate(vals):
                    out[v, kb::nvtk, jb::nvtk, ib::nvtk] = a.transpose(2, 1, 0)
    return out

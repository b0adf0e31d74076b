"""Initial conditions (host side, numpy).

These build the caller-owned state array ``Q(nx,ny,nz,nQ,nbasis)`` (Fortran
order, float64) that ``setup``/``step`` then advance.  They are fixtures for
the benchmark problems, not part of the hot path.  Where the reference has the
problem, the routine follows ``src/initialcon.f90`` line by line; only the
cell averages (basis function 1) are set, as there.
"""
from __future__ import annotations

import math

import numpy as np

from .config import Config, NQ

RH, MX, MY, MZ, EN, PXX, PYY, PZZ, PXY, PXZ, PYZ = range(NQ)


def empty_state(cfg: Config, dtype=np.float64) -> np.ndarray:
    return np.zeros(cfg.shape_f, dtype=dtype, order="F")


def cell_centres(cfg: Config):
    """params.f90:212-227 xc/yc/zc with the domain centred at the origin
    (initialize.f90:310-326): xc(i) = -lx/2 + (i - 1/2) dx, dx = 1/dxi,
    dxi = nx/lx."""
    dx, dy, dz = 1.0 / (cfg.nx / cfg.lx), 1.0 / (cfg.ny / cfg.ly), 1.0 / (cfg.nz / cfg.lz)
    xc = -cfg.lx / 2 + (np.arange(1, cfg.nx + 1) - 0.5) * dx
    yc = -cfg.ly / 2 + (np.arange(1, cfg.ny + 1) - 0.5) * dy
    zc = -cfg.lz / 2 + (np.arange(1, cfg.nz + 1) - 0.5) * dz
    return xc, yc, zc


def _background(cfg: Config) -> np.ndarray:
    """initialcon.f90:35-37: zero state with floor density and energy."""
    Q = empty_state(cfg)
    Q[:, :, :, RH, 0] = cfg.rh_floor
    Q[:, :, :, EN, 0] = cfg.T_floor * cfg.rh_floor / (cfg.aindex - 1.0)
    return Q


def _set_hydro(Q, dn, vx, vy, vz, pr, gamma):
    Q[:, :, :, RH, 0] = dn
    Q[:, :, :, MX, 0] = dn * vx
    Q[:, :, :, MY, 0] = dn * vy
    Q[:, :, :, MZ, 0] = dn * vz
    Q[:, :, :, EN, 0] = pr / (gamma - 1.0) + 0.5 * dn * (vx ** 2 + vy ** 2 + vz ** 2)


def sod(cfg: Config, p_hi: float = None, p_lo: float = None, rh_hi: float = 1.0, rh_lo: float = 0.125,
        ver: int = 0) -> np.ndarray:
    """initialcon.f90:190-235 sod_shock_tube_1d: high state where xc + yc <= 0
    (version 1) or xc <= 0 (version 0, the diaphragm at x = 0.5 of [0, 1]);
    pressures 1 and 0.1 times P_base."""
    p_hi = 1.0 * cfg.P_base if p_hi is None else p_hi
    p_lo = 0.1 * cfg.P_base if p_lo is None else p_lo
    Q = _background(cfg)
    xc, yc, zc = cell_centres(cfg)
    X = np.broadcast_to(xc[:, None, None], (cfg.nx, cfg.ny, cfg.nz))
    if ver == 1:
        X = X + np.broadcast_to(yc[None, :, None], (cfg.nx, cfg.ny, cfg.nz))
    left = X <= 0
    dn = np.where(left, rh_hi, rh_lo)
    pr = np.where(left, p_hi, p_lo)
    z = np.zeros_like(dn)
    _set_hydro(Q, dn, z, z, z, pr, cfg.aindex)
    return Q


def isentropic_vortex(cfg: Config, ver: int = 1, beta: float = 5.0) -> np.ndarray:
    """initialcon.f90:128-183 isentropic_vortex."""
    Q = _background(cfg)
    g = cfg.aindex
    aindm1 = g - 1.0
    vx_amb, vy_amb, Rgsqi = (1.0, 0.0, 1.0) if ver == 0 else (1.0, 1.0, 0.5)
    xc, yc, zc = cell_centres(cfg)
    X, Y = np.meshgrid(xc, yc, indexing="ij")
    X = np.broadcast_to(X[:, :, None], (cfg.nx, cfg.ny, cfg.nz))
    Y = np.broadcast_to(Y[:, :, None], (cfg.nx, cfg.ny, cfg.nz))
    r2 = X ** 2 + Y ** 2
    pi = math.pi
    dvx = -Y * beta / (2 * pi) * np.exp(Rgsqi * (1 - r2))
    dvy = X * beta / (2 * pi) * np.exp(Rgsqi * (1 - r2))
    dT = -(aindm1 * beta ** 2) / (16 * Rgsqi * g * pi ** 2) * np.exp(2 * Rgsqi * (1 - r2))
    vx, vy = vx_amb + dvx, vy_amb + dvy
    te = 1.0 + dT
    dn = te ** (1.0 / aindm1)
    pr = dn ** g
    _set_hydro(Q, dn, vx, vy, np.zeros_like(vx), pr, g)
    return Q


def isentropic_vortex_exact(cfg: Config, t: float, ver: int = 1, beta: float = 5.0, quad: int = 1) -> np.ndarray:
    """Density of the exactly advected vortex at time t (the IC shifted by the
    mean flow, periodically wrapped, initialcon.f90:158-177): sampled at the
    cell centres (quad = 1) or averaged over each cell by a quad x quad
    Gauss-Legendre rule (quad > 1), shape (nx, ny)."""
    vx_amb, vy_amb, Rgsqi = (1.0, 0.0, 1.0) if ver == 0 else (1.0, 1.0, 0.5)
    g = cfg.aindex
    xc, yc, zc = cell_centres(cfg)
    dx, dy = cfg.lx / cfg.nx, cfg.ly / cfg.ny
    if quad > 1:
        pts, wts = np.polynomial.legendre.leggauss(quad)
    else:
        pts, wts = np.zeros(1), np.full(1, 2.0)
    out = np.zeros((cfg.nx, cfg.ny))
    for a, wa in zip(pts, wts):
        for b, wb in zip(pts, wts):
            X, Y = np.meshgrid(xc + 0.5 * dx * a, yc + 0.5 * dy * b, indexing="ij")
            Xs = (X - vx_amb * t + cfg.lx / 2) % cfg.lx - cfg.lx / 2
            Ys = (Y - vy_amb * t + cfg.ly / 2) % cfg.ly - cfg.ly / 2
            r2 = Xs ** 2 + Ys ** 2
            dT = -((g - 1) * beta ** 2) / (16 * Rgsqi * g * math.pi ** 2) * np.exp(2 * Rgsqi * (1 - r2))
            out += 0.25 * wa * wb * (1.0 + dT) ** (1.0 / (g - 1))
    return out


def taylor_green(cfg: Config, rho: float = 1.0, V0: float = 1.0, perturb: float = 0.0, seed: int = 0) -> np.ndarray:
    """Taylor-Green vortex on [0, 2 pi]^3 (no reference IC): vx = V0 sin x cos y
    cos z, vy = -V0 cos x sin y cos z, vz = 0, rho = 1, p = colvis (= rho
    c^2/gamma), evaluated at cell centres shifted to [0, L).

    perturb > 0 adds seeded Gaussian noise of that amplitude to the velocity.
    The exact field has zero normal velocity on its symmetry planes, where
    the reference's HLLC with the stress-augmented point flux is
    discontinuous (the star fluxes differ by P_dd,L - P_dd,R at S_M = 0,
    flux.f90:87-89,623-643), so the unperturbed problem amplifies rounding
    differences to O(1e-6) within a few steps; the perturbation moves S_M
    off zero and makes trajectories comparable between implementations."""
    Q = _background(cfg)
    xc, yc, zc = cell_centres(cfg)
    x, y, z = xc + cfg.lx / 2, yc + cfg.ly / 2, zc + cfg.lz / 2
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    vx = V0 * np.sin(X) * np.cos(Y) * np.cos(Z)
    vy = -V0 * np.cos(X) * np.sin(Y) * np.cos(Z)
    vz = np.zeros_like(vx)
    if perturb > 0:
        rng = np.random.default_rng(seed)
        vx = vx + perturb * rng.standard_normal(vx.shape)
        vy = vy + perturb * rng.standard_normal(vx.shape)
        vz = vz + perturb * rng.standard_normal(vx.shape)
    p = cfg.colvis if cfg.colvis > 0 else 1.0
    _set_hydro(Q, np.full_like(vx, rho), vx, vy, vz, np.full_like(vx, p), cfg.aindex)
    return Q


def equilibrium(cfg: Config, rho: float = 1.0, T: float = 1.0) -> np.ndarray:
    """Uniform fluid at rest, p = rho T (fluctuating-hydro equilibrium)."""
    Q = _background(cfg)
    sh = (cfg.nx, cfg.ny, cfg.nz)
    z = np.zeros(sh)
    _set_hydro(Q, np.full(sh, rho), z, z, z, np.full(sh, rho * T), cfg.aindex)
    return Q


def channel(cfg: Config, amplitude: float = 1.0e-3, seed: int = 0, rho: float = 1.0, p: float = 1.0) -> np.ndarray:
    """Channel at rest plus a seeded Gaussian velocity perturbation of the
    given amplitude (cell averages of vx, vy).  No reference IC: the
    reference's poiseuille_flow (initialcon.f90:244-284) starts at rest and is
    driven by inflow."""
    Q = _background(cfg)
    rng = np.random.default_rng(seed)
    sh = (cfg.nx, cfg.ny, cfg.nz)
    vx = amplitude * rng.standard_normal(sh)
    vy = amplitude * rng.standard_normal(sh)
    _set_hydro(Q, np.full(sh, rho), vx, vy, np.zeros(sh), np.full(sh, p), cfg.aindex)
    return Q


def random_smooth(cfg: Config, seed: int = 0, amp: float = 0.05, stress_amp: float = 0.0) -> np.ndarray:
    """A positive, smooth-ish random state with all basis modes populated;
    used by parity tests to exercise every term of the operator."""
    rng = np.random.default_rng(seed)
    Q = equilibrium(cfg)
    nb = cfg.nbasis
    sh = (cfg.nx, cfg.ny, cfg.nz)
    Q[:, :, :, RH, 0] = 1.0 + amp * rng.standard_normal(sh)
    v = amp * rng.standard_normal((3,) + sh)
    Q[:, :, :, MX:MZ + 1, 0] = np.moveaxis(v * Q[:, :, :, RH, 0], 0, -1)
    Q[:, :, :, EN, 0] = (1.0 + amp * rng.standard_normal(sh)) / (cfg.aindex - 1) + \
        0.5 * (Q[:, :, :, MX, 0] ** 2 + Q[:, :, :, MY, 0] ** 2 + Q[:, :, :, MZ, 0] ** 2) / Q[:, :, :, RH, 0]
    if stress_amp > 0:
        Q[:, :, :, PXX:PYZ + 1, 0] = stress_amp * rng.standard_normal(sh + (6,))
    for b in range(1, nb):
        Q[:, :, :, :, b] = 0.1 * amp * rng.standard_normal(sh + (NQ,)) * np.abs(Q[:, :, :, :, 0]).mean(axis=(0, 1, 2))
    return Q


def ten_moment_stress(cfg: Config, Q: np.ndarray, p: float = 1.0, amp: float = 0.0, seed: int = 0) -> np.ndarray:
    """Fill the stress slots with the full second-moment tensor of the
    10-moment (ivis 2) form, P_ij = m_i m_j / rho + p delta_ij, plus seeded
    noise of amplitude amp, on the cell averages."""
    rng = np.random.default_rng(seed)
    rho = Q[:, :, :, RH, 0]
    m = [Q[:, :, :, MX, 0], Q[:, :, :, MY, 0], Q[:, :, :, MZ, 0]]
    for v, (a, b) in zip((PXX, PYY, PZZ, PXY, PXZ, PYZ), ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))):
        Q[:, :, :, v, 0] = m[a] * m[b] / rho + (p if a == b else 0.0) + amp * rng.standard_normal(rho.shape)
    return Q


# ---- the remaining problems of set_ic (initialcon.f90:41-69) ---------------
_M0, _M1, _W0, _W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
JET_TAG = 0x4A455400   # counter word 2 of the jet's uniforms


def philox_uniform(seed: int, site: np.ndarray, tag: int) -> np.ndarray:
    """Uniform numbers in [0, 1) from Philox-4x32-10 (Salmon et al., SC'11),
    counter (site_lo, site_hi, tag, 0), key = seed: the top 53 bits of the
    first two output words.  The device initialiser draws the same numbers."""
    mask = np.uint64(0xFFFFFFFF)
    site = np.asarray(site, dtype=np.uint64)
    c0, c1 = site & mask, site >> np.uint64(32)
    c2 = np.full_like(site, np.uint64(tag))
    c3 = np.zeros_like(site)
    k0, k1 = np.uint64(seed & 0xFFFFFFFF), np.uint64((seed >> 32) & 0xFFFFFFFF)
    for _ in range(10):
        p0 = np.uint64(_M0) * c0
        p1 = np.uint64(_M1) * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & mask
        hi1, lo1 = p1 >> np.uint64(32), p1 & mask
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0 = (k0 + np.uint64(_W0)) & mask
        k1 = (k1 + np.uint64(_W1)) & mask
    m = (c0 << np.uint64(21)) | (c1 >> np.uint64(11))
    return m.astype(np.float64) * (1.0 / 9007199254740992.0)


def hydro_jet(cfg: Config, seed: int = 0, beta: float = 1.0, beta2: float = 0.005) -> np.ndarray:
    """initialcon.f90:79-114 hydro_jet: dn = 1, T = T_floor, a jet
    m_x = beta dn / cosh(20 yc / lyu) with a random transverse kick
    beta2 (r - 1/2) / cosh(20 yc / lyu)^2, lyu = ly/2.  The reference draws r
    with Fortran's random_number (unseeded); here r comes from
    philox_uniform(seed, cell) so the state is reproducible."""
    Q = _background(cfg)
    xc, yc, zc = cell_centres(cfg)
    dn, te = 1.0, cfg.T_floor
    pr = te * dn
    cell = np.arange(cfg.nx * cfg.ny * cfg.nz, dtype=np.uint64).reshape(cfg.nz, cfg.ny, cfg.nx).transpose(2, 1, 0)
    rnum = philox_uniform(seed, cell, JET_TAG) - 0.5
    lyu = cfg.ly / 2.0
    ch = np.broadcast_to(np.cosh(20 * yc / lyu)[None, :, None], (cfg.nx, cfg.ny, cfg.nz))
    smx = beta * dn / ch
    smy = beta2 * rnum / ch ** 2
    Q[:, :, :, RH, 0] = dn
    Q[:, :, :, MX, 0] = smx
    Q[:, :, :, MY, 0] = smy
    Q[:, :, :, MZ, 0] = 0.0
    Q[:, :, :, EN, 0] = pr / (cfg.aindex - 1.0) + 0.5 * (smx ** 2 + smy ** 2 + 0.0 ** 2) / dn
    return Q


def fluid_at_rest(cfg: Config) -> np.ndarray:
    """initialcon.f90:244-361 poiseuille_flow / pipe_cylinder_2d: dn = 1,
    T = T_floor, v = 0 (their inflow and cylinder boundary arrays are never
    applied by the reference's step)."""
    Q = _background(cfg)
    z = np.zeros((cfg.nx, cfg.ny, cfg.nz))
    _set_hydro(Q, z + 1.0, z, z, z, z + cfg.T_floor, cfg.aindex)
    return Q


def from_icid(cfg: Config, icid: int, seed: int = 0) -> np.ndarray:
    """set_ic (initialcon.f90:20-72) by problem id."""
    if icid == 0:
        return hydro_jet(cfg, seed)
    if icid in (1, 2):
        return isentropic_vortex(cfg, icid - 1)
    if icid in (3, 4):
        return sod(cfg, ver=icid - 3)
    if icid in (5, 6, 7):
        return fluid_at_rest(cfg)
    raise ValueError(f"unknown icid {icid}")

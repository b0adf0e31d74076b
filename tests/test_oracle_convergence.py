"""Order of accuracy of the oracle on a smooth solution: a density wave
rho = 1 + 0.2 sin(2 pi x) carried at u = 1 under p = 1 is an exact solution of
the Euler equations, back at its start after one period.  The error of the
discontinuous-Galerkin solution in L2 then falls as h^(p+1) with the degree p
of the basis in x: second order for the linear families (nb 4, 8), third for
the quadratic one (nb 10), with SSP-RK3 at a time step small enough that the
spatial error dominates.  A wrong quadrature weight, basis normalisation,
face table or flux term drops the order (to one or less), so this checks the
tables, the volume and surface integrals and the integrator of the
restatement (basis_funcs.f90:265-627, flux.f90:700-930, integrator.f90:62-122)
against the method's defining property rather than against themselves.
(The wave is a contact: HLLC and Roe resolve it exactly at each face, so
their errors agree to rounding; the central/LLF flux adds dissipation of the
same order.)  Measured: nb 4 errors 1.25e-3, 2.77e-4, 6.65e-5 on 16, 32, 64
cells (rates 2.18, 2.06); nb 10 2.58e-4, 3.20e-5, 3.99e-6 on 8, 16, 32 (3.01,
3.00).

The state is the L2 projection onto the reference's unnormalised Legendre
modes (P0 = 1, P1 = s, P2 = 1.5 s^2 - 0.5 on s in [-1, 1], mass 1/(2k+1)):
c_k = (2k + 1)/2 * integral of f P_k ds, by an 8-point Gauss rule per cell."""
import math

import numpy as np
import pytest

from hermeshd_gb300 import config

RH, MX, EN = 0, 1, 4
# index of the x-modes P1(x), P2(x) in each family (initialize.f90:126-194)
XMODES = {4: {1: 1}, 8: {1: 1}, 10: {1: 1, 2: 7}}


def _legendre(k, s):
    return [np.ones_like(s), s, 1.5 * s * s - 0.5][k]


def project(cfg, f):
    """Modal coefficients (nx, nmodes) of f(x) on the cells of [-lx/2, lx/2]."""
    nx, dx = cfg.nx, cfg.lx / cfg.nx
    s, w = np.polynomial.legendre.leggauss(8)
    xc = -cfg.lx / 2 + dx * (np.arange(nx) + 0.5)
    fx = f(xc[:, None] + 0.5 * dx * s[None, :])
    deg = max(XMODES[cfg.nbasis])
    return np.stack([(2 * k + 1) / 2 * (fx * _legendre(k, s)[None, :]) @ w for k in range(deg + 1)], axis=1)


def set_state(cfg, Q, c):
    """rho from its coefficients; m_x = rho u and E = p/(gamma-1) + rho u^2 / 2
    are affine in rho, so their coefficients follow exactly."""
    Q[...] = 0.0
    modes = {0: 0, **XMODES[cfg.nbasis]}
    for k, m in modes.items():
        Q[:, 0, 0, RH, m] = c[:, k]
        Q[:, 0, 0, MX, m] = c[:, k]                                # u = 1
        Q[:, 0, 0, EN, m] = 0.5 * c[:, k]
    Q[:, 0, 0, EN, 0] += 1.0 / (cfg.aindex - 1)                    # p = 1


def l2_error(cfg, Q, c):
    """L2 norm over the line of rho_h - rho_exact(projected); the projection
    error of the exact solution is of the same order, so this carries the order."""
    dx = cfg.lx / cfg.nx
    modes = {0: 0, **XMODES[cfg.nbasis]}
    e2 = 0.0
    for k, m in modes.items():
        e2 += float(((Q[:, 0, 0, RH, m] - c[:, k]) ** 2).sum()) * dx / (2 * k + 1)
    return math.sqrt(e2)


def run(nb, iq, ihllc, nx):
    import oracle as O
    cfg = config.Config(nx=nx, ny=1, nz=1, nbasis=nb, iquad=iq, ivis=0, coll=0.0, colvis=0.0, ihllc=ihllc,
                        iorder=3, lx=1.0, ly=1.0 / nx, lz=1.0 / nx)
    c = project(cfg, lambda x: 1.0 + 0.2 * np.sin(2 * math.pi * x))
    Q = np.zeros(cfg.shape_f, order="F")
    set_state(cfg, Q, c)
    smax = 1.0 + math.sqrt(cfg.aindex / 0.8)                       # |u| + c at the density minimum
    dx = cfg.lx / nx
    n = int(math.ceil(1.0 / (0.1 * dx / smax)))                    # one period, Courant number 0.1
    m0 = Q[:, 0, 0, RH, 0].sum()
    O.Oracle(cfg).advance_fixed_dt(Q, 1.0 / n, n)
    return l2_error(cfg, Q, c), Q[:, 0, 0, RH, 0].sum() / m0


@pytest.mark.parametrize("nb,iq,ihllc,grids,order", [
    (4, 2, 1, (16, 32, 64), 1.8),        # linear in x, HLLC
    (4, 2, 2, (16, 32, 64), 1.8),        # linear in x, Roe
    (8, 2, 0, (16, 32, 64), 1.8),        # the bilinear family, central/LLF flux
    (10, 3, 1, (8, 16, 32), 2.7),        # quadratic in x, HLLC
], ids=["nb4_hllc", "nb4_roe", "nb8_central", "nb10_hllc"])
def test_smooth_wave_converges_at_the_basis_order(nb, iq, ihllc, grids, order):
    errs = []
    for nx in grids:
        e, mass = run(nb, iq, ihllc, nx)
        assert abs(mass - 1.0) < 1e-12                              # mass conserved to rounding over ~3000 steps
        errs.append(e)
    rates = [math.log2(errs[i] / errs[i + 1]) for i in range(len(errs) - 1)]
    assert min(rates) >= order, (errs, rates)
    assert max(rates) <= order + 1.6, (errs, rates)                # not a smaller-than-expected error by accident

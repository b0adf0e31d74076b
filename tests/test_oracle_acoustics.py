"""A small-amplitude sound wave in the oracle: a right-moving acoustic wave on
a periodic line travels at c = sqrt(gamma p / rho), so after half a period the
density perturbation is the negative of the initial one and after a full
period it is back, to the scheme's accuracy (second order for the linear
basis, third for the quadratic one) -- the Euler fluxes, HLLC and the SSP-RK
integrator of the restatement against the linearised physics."""
import math

import numpy as np
import pytest

from hermeshd_gb300 import config

RH, MX, EN = 0, 1, 4


def acoustic_wave(cfg, eps=1e-4, rho0=1.0, p0=1.0):
    g = cfg.aindex
    c = math.sqrt(g * p0 / rho0)
    Q = np.zeros(cfg.shape_f, order="F")
    dx = cfg.lx / cfg.nx
    xl = -cfg.lx / 2 + dx * np.arange(cfg.nx)            # cell left edges (domain centred on 0)
    k = 2 * math.pi / cfg.lx
    # exact cell averages of sin(k x)
    s = (np.cos(k * xl) - np.cos(k * (xl + dx))) / (k * dx)
    rho = rho0 + eps * s
    u = eps * c * s / rho0
    p = p0 + eps * c * c * s
    Q[:, 0, 0, RH, 0] = rho
    Q[:, 0, 0, MX, 0] = rho * u
    Q[:, 0, 0, EN, 0] = p / (g - 1) + 0.5 * rho * u * u
    return Q, c, eps


@pytest.mark.parametrize("nb,iq,nx,tol", [(4, 2, 64, 5e-3), (10, 3, 32, 5e-3)])
def test_sound_wave_travels_at_the_sound_speed(nb, iq, nx, tol):
    import oracle as O
    cfg = config.Config(nx=nx, ny=1, nz=1, nbasis=nb, iquad=iq, ivis=0, coll=0.0, colvis=0.0, ihllc=1, iorder=3,
                        lx=1.0, ly=1.0 / nx, lz=1.0 / nx)
    Q, c, eps = acoustic_wave(cfg)
    d0 = Q[:, 0, 0, RH, 0] - 1.0
    period = cfg.lx / c
    n = int(math.ceil(period / (0.1 * (cfg.lx / nx) / c)))
    n += n % 2
    dt = period / n
    orc = O.Oracle(cfg)
    orc.advance_fixed_dt(Q, dt, n // 2)
    half = Q[:, 0, 0, RH, 0] - 1.0
    assert np.linalg.norm(half + d0) <= tol * np.linalg.norm(d0), np.linalg.norm(half + d0) / np.linalg.norm(d0)
    orc.advance_fixed_dt(Q, dt, n // 2)
    full = Q[:, 0, 0, RH, 0] - 1.0
    err = np.linalg.norm(full - d0) / np.linalg.norm(d0)
    assert err <= tol, err
    # a wave at the wrong speed would be out of phase: one at 0.9 c is off by ~0.6
    assert np.linalg.norm(np.roll(d0, nx // 10) - d0) / np.linalg.norm(d0) > 20 * tol

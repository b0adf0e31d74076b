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


@pytest.mark.parametrize("ihllc", [2, 0])
def test_shear_wave_decays_at_the_navier_stokes_rate(ihllc):
    """ivis 1 with coll = p / mu and colvis = p relaxes the stress to the
    Navier-Stokes shear stress -mu dv/dx: a transverse velocity sin(k x) decays
    as exp(-mu k^2 t / rho) (relaxation time mu / p = 0.01 here, so the
    10-moment correction is ~0.4 %).  With the Roe and the central flux; the
    reference's HLLC receives the stress-augmented point flux and is
    discontinuous at S_M = 0, where a shear wave (v_x = 0) sits at every face,
    and it amplifies the wave instead (flux.f90:87-89,623-643)."""
    import oracle as O
    nx, mu, p0, rho0, eps = 64, 0.01, 1.0, 1.0, 1e-3
    cfg = config.Config(nx=nx, ny=1, nz=1, nbasis=4, iquad=2, ivis=1, coll=p0 / mu, colvis=p0, ihllc=ihllc, iorder=3,
                        lx=1.0, ly=1.0 / nx, lz=1.0 / nx)
    dx = cfg.lx / nx
    xl = -cfg.lx / 2 + dx * np.arange(nx)
    k = 2 * math.pi / cfg.lx
    s = (np.cos(k * xl) - np.cos(k * (xl + dx))) / (k * dx)
    Q = np.zeros(cfg.shape_f, order="F")
    Q[:, 0, 0, RH, 0] = rho0
    Q[:, 0, 0, 2, 0] = rho0 * eps * s                          # m_y
    Q[:, 0, 0, EN, 0] = p0 / (cfg.aindex - 1) + 0.5 * rho0 * (eps * s) ** 2
    orc = O.Oracle(cfg)
    t = 0.0
    while t < 1.0:
        t, _ = orc.advance(Q, 20, t=t)
    amp = float(Q[:, 0, 0, 2, 0] @ s) / float(rho0 * eps * (s @ s))
    expect = math.exp(-mu * k * k * t / rho0)
    assert abs(amp / expect - 1.0) < 0.01, (amp, expect, t)


@pytest.mark.parametrize("ihllc", [0, 1])
def test_tait_sound_wave_travels_at_the_linearised_speed(ihllc):
    """ieos 2: P = (gamma-1)(E - rho v^2/2) + P_1 (rho^7.2 - 1) + P_base with the
    energy flux (E + P) v; linearised at rest, c^2 = ((gamma-1)(E0 + P0) +
    7.2 P_1 rho0^7.2) / rho0.  A right-moving wave of that speed returns after
    a period, with the central flux and with the reference's HLLC (its stale
    1/rho only shifts the wave-speed estimates, flux.f90:533-534)."""
    import oracle as O
    nx = 64
    cfg = config.Config(nx=nx, ny=1, nz=1, nbasis=4, iquad=2, ivis=0, coll=0.0, colvis=0.0, ihllc=ihllc, iorder=3,
                        ieos=2, P_1=0.05, P_base=1.0, lx=1.0, ly=1.0 / nx, lz=1.0 / nx)
    g, rho0, pig0, eps = cfg.aindex, 1.0, 1.0, 1e-4
    E0 = pig0 / (g - 1)
    P0 = pig0 + cfg.P_1 * (rho0 ** 7.2 - 1) + cfg.P_base
    c2 = ((g - 1) * (E0 + P0) + 7.2 * cfg.P_1 * rho0 ** 7.2) / rho0
    c = math.sqrt(c2)
    dx = cfg.lx / nx
    xl = -cfg.lx / 2 + dx * np.arange(nx)
    k = 2 * math.pi / cfg.lx
    s = (np.cos(k * xl) - np.cos(k * (xl + dx))) / (k * dx)
    rho, u = rho0 + eps * s, eps * c * s / rho0
    dE = (eps * c2 * s - 7.2 * cfg.P_1 * rho0 ** 6.2 * eps * s) / (g - 1)
    Q = np.zeros(cfg.shape_f, order="F")
    Q[:, 0, 0, RH, 0] = rho
    Q[:, 0, 0, MX, 0] = rho * u
    Q[:, 0, 0, EN, 0] = E0 + dE + 0.5 * rho * u * u
    d0 = Q[:, 0, 0, RH, 0] - rho0
    period = cfg.lx / c
    n = int(math.ceil(period / (0.1 * dx / c)))
    n += n % 2
    orc = O.Oracle(cfg)
    orc.advance_fixed_dt(Q, period / n, n // 2)
    assert np.linalg.norm(Q[:, 0, 0, RH, 0] - rho0 + d0) <= 5e-3 * np.linalg.norm(d0)
    orc.advance_fixed_dt(Q, period / n, n // 2)
    assert np.linalg.norm(Q[:, 0, 0, RH, 0] - rho0 - d0) <= 5e-3 * np.linalg.norm(d0)

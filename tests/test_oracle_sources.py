"""The oracle's sources (sources.f90:12-84) against their formulas on uniform
periodic states, where the surface and volume terms of the cell average
vanish and the right-hand side of coefficient 0 is minus the source:
ivis 0 relaxes the stresses, -coll P_ij (:37-43), so R = coll P_ij; ivis 1
has none (the relaxation is in the update's factor); ivis 2 drives the
10-moment stresses with coll rho (v_i v_j - delta_ij |v|^2 / 3) (:51-69);
the hydro rows have no source (R = 0).  Higher coefficients of a uniform
state stay at rounding level."""
import numpy as np
import pytest

from hermeshd_gb300 import config

RH, MX, MY, MZ, EN, PXX, PYY, PZZ, PXY, PXZ, PYZ = range(11)


def uniform_state(cfg, rho=1.3, v=(0.4, -0.25, 0.15), p=1.1, stress=(0.9, 1.2, 0.7, 0.05, -0.08, 0.11)):
    Q = np.zeros(cfg.shape_f, order="F")
    Q[..., RH, 0] = rho
    for k in range(3):
        Q[..., MX + k, 0] = rho * v[k]
    Q[..., EN, 0] = p / (cfg.aindex - 1.0) + 0.5 * rho * (v[0] ** 2 + v[1] ** 2 + v[2] ** 2)
    for m, s in enumerate(stress):
        Q[..., PXX + m, 0] = s
    return Q


@pytest.mark.parametrize("ivis", [0, 1, 2])
@pytest.mark.parametrize("nb,iq", [(4, 2), (10, 3)])
def test_uniform_state_rhs_is_minus_the_source(ivis, nb, iq):
    import oracle as O
    coll = 1.7
    cfg = config.Config(nx=3, ny=2, nz=2, nbasis=nb, iquad=iq, ivis=ivis, coll=coll, colvis=0.6)
    Q = uniform_state(cfg)
    R = O.Oracle(cfg).rhs(np.asfortranarray(Q), limit=False)
    rho = Q[0, 0, 0, RH, 0]
    v = Q[0, 0, 0, MX:MZ + 1, 0] / rho
    P = Q[0, 0, 0, PXX:PYZ + 1, 0]
    if ivis == 0:
        expect = coll * P
    elif ivis == 1:
        expect = np.zeros(6)
    else:
        v2 = float(v @ v)
        pairs = ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))
        expect = -np.array([coll * rho * (v[i] * v[j] - (v2 / 3.0 if i == j else 0.0)) for i, j in pairs])
    scale = np.abs(Q).max()
    for cell in np.ndindex(cfg.nx, cfg.ny, cfg.nz):
        r0 = R[cell + (slice(None), 0)]
        assert np.allclose(r0[RH:EN + 1], 0.0, atol=1e-13 * scale), r0[:5]
        assert np.allclose(r0[PXX:], expect, rtol=1e-13, atol=1e-13 * scale), (r0[PXX:], expect)
        assert np.abs(R[cell + (slice(None), slice(1, None))]).max() <= 1e-12 * scale


def test_ten_moment_stage_relaxes_the_deviator_and_keeps_the_trace():
    """ivis 2's semi-implicit update (integrator.f90:207-224) of a uniform state
    at rest: the pressure tensor's trace (3 p) is kept and its deviator scaled
    by faci = 1 / (1 + dt coll) per stage; the off-diagonal stresses likewise."""
    import oracle as O
    coll, dt = 3.0, 0.05
    cfg = config.Config(nx=2, ny=2, nz=2, nbasis=4, iquad=2, ivis=2, coll=coll, colvis=1.0)
    Q = uniform_state(cfg, v=(0.0, 0.0, 0.0), stress=(1.3, 0.9, 0.8, 0.07, -0.05, 0.02))
    E = O.Oracle(cfg).euler_step(np.asfortranarray(Q), dt)
    faci = 1.0 / (1.0 + dt * coll)
    P0, P1 = Q[0, 0, 0, PXX:PYZ + 1, 0], E[0, 0, 0, PXX:PYZ + 1, 0]
    assert P1[:3].sum() == pytest.approx(P0[:3].sum(), rel=1e-14)
    dev0, dev1 = P0[:3] - P0[:3].mean(), P1[:3] - P1[:3].mean()
    assert np.allclose(dev1, faci * dev0, rtol=1e-13, atol=1e-15)
    assert np.allclose(P1[3:], faci * P0[3:], rtol=1e-13, atol=1e-15)

"""Initial states of set_ic (initialcon.f90:20-361): the host restatement
(ic.from_icid) on the CPU, and the device initialiser (hermes_init_state)
against it on the GPU.

Tolerance of the device states: 4e-16 relative to each variable's largest
cell average in FP64 (exp, pow and cosh of CUDA and of the host libm differ
in the last bit or two); the FP32 states are the FP64 values rounded, to one
float32 ulp."""
import numpy as np
import pytest

from hermeshd_gb300 import config, ic


def test_philox_uniforms_match_the_oracle_generator():
    import oracle as O
    for site in (0, 5, 2 ** 33 + 7):
        w = O.philox4x32_10([site & 0xFFFFFFFF, site >> 32, ic.JET_TAG, 0], [123, 0])
        u = ((w[0] << 21) | (w[1] >> 11)) * 2.0 ** -53
        assert ic.philox_uniform(123, np.array([site]), ic.JET_TAG)[0] == u


def test_host_states():
    cfg = config.Config(nx=8, ny=6, nz=1, nbasis=4, iquad=2, lx=2.0, ly=2.0, P_base=2.0)
    s1 = ic.from_icid(cfg, 4)
    xc, yc, _ = ic.cell_centres(cfg)
    hi = (xc[:, None] + yc[None, :]) <= 0
    assert np.array_equal(s1[:, :, 0, 0, 0] == 1.0, hi)
    assert np.allclose(s1[:, :, 0, 4, 0][hi], 2.0 / (cfg.aindex - 1))
    j1, j2 = ic.from_icid(cfg, 0, seed=3), ic.from_icid(cfg, 0, seed=3)
    assert np.array_equal(j1, j2) and not np.array_equal(j1, ic.from_icid(cfg, 0, seed=4))
    r = ic.from_icid(cfg, 6)
    assert np.all(r[:, :, :, 0, 0] == 1.0) and np.all(r[:, :, :, 1:4, 0] == 0.0)


CASES = [(config.Config(nx=16, ny=12, nz=2, nbasis=4, iquad=2, lx=10.0, ly=8.0, lz=1.0), icid)
         for icid in range(8)] + [
    (config.Config(nx=12, ny=12, nz=1, nbasis=10, iquad=3, lx=10.0, ly=10.0), 2),
    (config.Config(nx=12, ny=12, nz=1, nbasis=10, iquad=3, lx=10.0, ly=10.0, precision="fp32"), 2),
    (config.Config(nx=16, ny=8, nz=1, nbasis=8, iquad=2, lx=1.0, ly=0.5, precision="fp32"), 0),
]


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(len(CASES)))
def test_device_initial_state_matches_host(k):
    import torch
    from hermeshd_gb300.solver import Solver
    cfg, icid = CASES[k]
    s = Solver(cfg)
    q = torch.full(cfg.shape_c, 7.0, dtype=s.dtype, device=s.device)    # every coefficient overwritten
    s.init_state(q, icid, seed=11)
    got = s.to_numpy(q)
    want = ic.from_icid(cfg, icid, seed=11)
    if cfg.precision == "fp32":
        want = want.astype(np.float32).astype(np.float64)
        tol = 2.0 ** -23
    else:
        tol = 4e-16
    assert np.array_equal(got[..., 1:], want[..., 1:])
    for v in range(11):
        scale = max(np.abs(want[..., v, 0]).max(), 1e-300)
        assert np.abs(got[..., v, 0] - want[..., v, 0]).max() <= tol * scale, (icid, v)


@pytest.mark.gpu
def test_device_initial_state_of_an_ensemble():
    from hermeshd_gb300.solver import Ensemble
    base = config.Config(nx=8, ny=8, nz=1, nbasis=4, iquad=2)
    dims = [(8, 8, 1), (6, 10, 1), (12, 4, 1)]
    lengths = [(10.0, 10.0, 1.0), (6.0, 11.0, 1.0), (9.0, 3.0, 1.0)]
    ens = Ensemble(base, dims, lengths, seeds=[0, 1, 2])
    q = ens.new_state()
    ens.init_state(q, 2)
    for i, ((nx, ny, nz), (lx, ly, lz)) in enumerate(zip(dims, lengths)):
        c = base.replace(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz)
        want = ic.from_icid(c, 2)
        got = np.asfortranarray(ens.box_view(q, i).cpu().numpy().T)
        assert np.array_equal(got[..., 1:], want[..., 1:])
        for v in range(11):
            scale = max(np.abs(want[..., v, 0]).max(), 1e-300)
            assert np.abs(got[..., v, 0] - want[..., v, 0]).max() <= 4e-16 * scale, (i, v)

"""FP64 conservation sums (hermes_conserved) of FP64 and FP32 states, single
grids and ensembles: against numpy sums of the cell averages, the same bits on
every call, and conservation by the periodic step."""
import numpy as np
import pytest

from hermeshd_gb300 import config, ic

pytestmark = pytest.mark.gpu


def _ref(Qf, cfg):
    vol = (1.0 / (cfg.nx / cfg.lx)) * (1.0 / (cfg.ny / cfg.ly)) * (1.0 / (cfg.nz / cfg.lz))
    return np.array([Qf[:, :, :, v, 0].astype(np.float64).sum() for v in range(5)])


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_sums_match_numpy_and_repeat_bitwise(prec):
    from hermeshd_gb300.solver import Solver
    cfg = config.Config(nx=40, ny=30, nz=20, nbasis=4, iquad=2, lx=2.0, ly=1.5, lz=1.0, precision=prec)
    Q = ic.random_smooth(cfg, seed=1, amp=0.1)
    s = Solver(cfg)
    q = s.from_numpy(Q)
    a = s.conserved(q)
    b = s.conserved(q)
    assert np.array_equal(a, b)
    vol = (1.0 / (cfg.nx / cfg.lx)) * (1.0 / (cfg.ny / cfg.ly)) * (1.0 / (cfg.nz / cfg.lz))
    want = _ref(s.to_numpy(q), cfg) * vol
    assert np.allclose(a[0], want, rtol=1e-13, atol=1e-13 * np.abs(want).max())


def test_ensemble_sums_per_box():
    from hermeshd_gb300.solver import Ensemble
    base = config.fh_box(8, precision="fp32", seed=0)
    dims = [(8, 8, 8), (12, 12, 12), (30, 30, 30)]
    dx = base.lx / 8
    ens = Ensemble(base, dims, [(n * dx,) * 3 for (n, _, _) in dims], seeds=[0, 1, 2])
    q = ens.new_state()
    ens.init_state(q, 6)
    s = ens.conserved(q)
    for i, (n, _, _) in enumerate(dims):
        vol_total = (n * dx) ** 3
        assert s[i, 0] == pytest.approx(vol_total, rel=1e-12)
        assert s[i, 4] == pytest.approx(vol_total * base.T_floor / (base.aindex - 1.0), rel=1e-6)


def test_periodic_step_conserves():
    from hermeshd_gb300.solver import Solver
    cfg = config.isentropic_vortex_2d(n=32)
    s = Solver(cfg)
    q, q1 = s.from_numpy(ic.isentropic_vortex(cfg)), s.new_state()
    c0 = s.conserved(q)
    s.advance(q, q1, 20)
    c1 = s.conserved(q)
    assert np.all(np.abs(c1 - c0) <= 1e-12 * np.abs(c0).max())

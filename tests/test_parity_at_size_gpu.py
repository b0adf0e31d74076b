"""GPU parity at the benchmarked sizes (the headline grid and the 3-D
Taylor-Green grid), through the C ABI, against the FP64 oracle run on the
host cores over the same steps.

  2-D isentropic vortex 128 x 128, nbasis 10, HLLC, SSP-RK3, 100 steps:
      FP64 path within 1e-11 relative L2, time within 1e-13;
      FP32 path within 1e-5 of the FP64 oracle.
  3-D Taylor-Green 64^3, ivis 1, nbasis 4, SSP-RK3 (symmetry broken by 1e-3,
  as in the step-parity case): 10 steps, FP64 within 1e-11, FP32 within 1e-5.

The oracle's runs take about 10 s each on 16 host cores."""
import numpy as np
import pytest

from hermeshd_gb300 import config, ic
from helpers import rel_l2

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-11
FP32_TOL = 1e-5


def _oracle_run(cfg, Q0, steps):
    import oracle as O
    Qo = Q0.copy(order="F")
    t, _ = O.Oracle(cfg).advance(Qo, steps)
    return Qo, t


def _gpu_run(cfg, Q0, steps):
    from hermeshd_gb300.solver import Solver
    s = Solver(cfg)
    q, q1 = s.from_numpy(Q0), s.new_state()
    t, _ = s.advance(q, q1, steps)
    out = s.to_numpy(q)
    s.close()
    return out, t


@pytest.fixture(scope="module")
def vortex128():
    cfg = config.isentropic_vortex_2d(n=128)
    Q0 = ic.isentropic_vortex(cfg)
    Qo, to = _oracle_run(cfg, Q0, 100)
    return cfg, Q0, Qo, to


@pytest.fixture(scope="module")
def tgv64():
    cfg = config.taylor_green_3d(n=64, precision="fp64")
    Q0 = ic.taylor_green(cfg, perturb=1e-3, seed=1)
    Qo, to = _oracle_run(cfg, Q0, 10)
    return cfg, Q0, Qo, to


def test_vortex128_nb10_100_steps_fp64(vortex128):
    cfg, Q0, Qo, to = vortex128
    g, t = _gpu_run(cfg, Q0, 100)
    assert abs(t - to) <= 1e-13 * to
    err = rel_l2(g, Qo)
    assert err < STEP_TOL, f"rel L2 {err:.3e}"


def test_vortex128_nb10_100_steps_fp32_vs_fp64_oracle(vortex128):
    cfg, Q0, Qo, to = vortex128
    g, t = _gpu_run(cfg.replace(precision="fp32"), Q0, 100)
    assert abs(t - to) <= 1e-6 * to      # the CFL reduction is FP64 on FP32 states
    err = rel_l2(g, Qo)
    assert err < FP32_TOL, f"rel L2 {err:.3e}"


def test_tgv64_ivis1_10_steps_fp64(tgv64):
    cfg, Q0, Qo, to = tgv64
    g, t = _gpu_run(cfg, Q0, 10)
    assert abs(t - to) <= 1e-13 * to
    err = rel_l2(g, Qo)
    assert err < STEP_TOL, f"rel L2 {err:.3e}"


def test_tgv64_ivis1_10_steps_fp32_vs_fp64_oracle(tgv64):
    cfg, Q0, Qo, to = tgv64
    g, t = _gpu_run(cfg.replace(precision="fp32"), Q0, 10)
    err = rel_l2(g, Qo)
    assert err < FP32_TOL, f"rel L2 {err:.3e}"

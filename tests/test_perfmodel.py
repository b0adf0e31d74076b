"""The algorithmic cost model behind the roofline figures: bytes per DOF and
stage (2s per plain stage, 3s with Q^n folded in; RK2 2.5s, RK3 8s/3) and the
flop count of the benchmarked vortex stage, which bench.py's alu block and the
executed-flop comparison are quoted against."""
import pytest

from hermeshd_gb300 import config, perfmodel


def test_bytes_per_dof_stage():
    assert perfmodel.bytes_per_dof_stage("fp64", 2) == 20.0
    assert perfmodel.bytes_per_dof_stage("fp32", 2) == 10.0
    assert perfmodel.bytes_per_dof_stage("fp64", 3) == pytest.approx(64.0 / 3.0)
    assert perfmodel.bytes_per_dof_stage("fp32", 3) == pytest.approx(32.0 / 3.0)


def test_vortex_flops_per_cell_stage():
    f = perfmodel.flops_per_cell_stage(config.isentropic_vortex_2d(n=128))
    assert f["total"] == pytest.approx(41147.67, abs=0.01)
    assert f["face"] == 14955 and f["cell"] == 26071
    assert sum(v for k, v in f.items() if k != "total") == pytest.approx(f["total"])
    # the linear basis costs a fraction of the quadratic one
    f4 = perfmodel.flops_per_cell_stage(config.taylor_green_3d(n=8))
    assert f4["total"] < 0.3 * f["total"]

"""The fused stage (k_tile, dg_tile.cuh: one kernel per SSP-RK stage of the
linear basis over tiles of 8 x 8 x 4 cells, the CFL reduction fused with the
first stage's limiter, each stage's output limited for the next stage)
against the FP64 oracle, through the C ABI:

  one right-hand side (hermes_rhs, fused stage forced on) for every nbasis-4
  ivis 0/1 right-hand-side case of the parity suite, including grids that
  fill no tile and 2-D grids                                  1e-12
  steps of Taylor-Green, walls, noisy fluctuating hydro, body force   1e-11
  FP32 against the FP64 oracle                                1e-5
and, among its own runs, the same bits: an ensemble equals its boxes run
alone, and one or several steps per CUDA graph give the same state.
The fused and separate-kernel paths agree to rounding (1e-13)."""
import numpy as np
import pytest

from hermeshd_gb300 import config, ic
from helpers import rel_l2
from test_parity_gpu import RHS_CASES

pytestmark = pytest.mark.gpu

RHS_TOL, STEP_TOL, FP32_TOL = 1e-12, 1e-11, 1e-5

TILE_RHS = sorted(k for k, (c, _) in RHS_CASES.items() if c.nbasis == 4 and c.ivis < 2)


def _solver(cfg, tile=1):
    from hermeshd_gb300.solver import Solver
    s = Solver(cfg)
    s.set_launch(tile_stage=tile)
    assert s.get_launch()["tile_stage"] == tile
    return s


@pytest.mark.parametrize("name", TILE_RHS)
def test_tile_rhs_parity(name):
    import oracle as O
    cfg, stress = RHS_CASES[name]
    Q = ic.random_smooth(cfg, seed=7, amp=0.1, stress_amp=0.05 * stress)
    Qo = Q.copy(order="F")
    r_o = O.Oracle(cfg).rhs(Qo, limit=True)
    s = _solver(cfg)
    q = s.from_numpy(Q)
    r_g = s.to_numpy(s.rhs(q, limit=True))
    assert rel_l2(s.to_numpy(q), Qo) < RHS_TOL
    err = rel_l2(r_g, r_o)
    assert err < RHS_TOL, f"{name}: rel L2 {err:.3e}"


STEP_CASES = {
    "tgv_12_rk3_ivis1": (lambda: config.taylor_green_3d(n=12, precision="fp64"),
                         lambda c: ic.taylor_green(c, perturb=1e-3, seed=1), 30),
    "walls_ivis1_rk2": (lambda: config.Config(nx=10, ny=9, nz=6, nbasis=4, iquad=2, ivis=1, coll=2.0, colvis=0.5,
                                              xlobc="wall", xhibc="noslip", ylobc="noslip", yhibc="wall",
                                              zlobc="outflow", zhibc="wall"),
                        lambda c: ic.random_smooth(c, seed=5, amp=0.05, stress_amp=0.01), 30),
    "fh_noise_16_rk2": (lambda: config.fh_box(16, precision="fp64", seed=42), lambda c: ic.equilibrium(c), 30),
    "ivis0_relax_rk3_roe": (lambda: config.Config(nx=9, ny=8, nz=5, nbasis=4, iquad=2, ivis=0, coll=0.7, ihllc=2),
                            lambda c: ic.random_smooth(c, seed=3, amp=0.05, stress_amp=0.02), 30),
    "bodyforce_noslip_2d": (lambda: config.Config(nx=8, ny=12, nz=1, nbasis=4, iquad=2, ivis=1, coll=5.0,
                                                  colvis=1.0, ylobc="noslip", yhibc="noslip", body_force=0.1),
                            lambda c: ic.random_smooth(c, seed=4, amp=0.02), 30),
}


@pytest.mark.parametrize("name", sorted(STEP_CASES))
def test_tile_steps_parity(name):
    import oracle as O
    mk, ic0, steps = STEP_CASES[name]
    cfg = mk()
    Q0 = ic0(cfg)
    Qo = Q0.copy(order="F")
    to, _ = O.Oracle(cfg).advance(Qo, steps)
    s = _solver(cfg)
    q, q1 = s.from_numpy(Q0), s.new_state()
    t, _ = s.advance(q, q1, steps)
    assert abs(t - to) <= 1e-13 * to
    err = rel_l2(s.to_numpy(q), Qo)
    assert err < STEP_TOL, f"{name}: rel L2 {err:.3e}"
    s.close()


@pytest.mark.parametrize("name", ["tgv_12_rk3_ivis1", "fh_noise_16_rk2"])
def test_tile_fp32_vs_fp64_oracle(name):
    import oracle as O
    mk, ic0, steps = STEP_CASES[name]
    cfg = mk()
    Q0 = ic0(cfg)
    Qo = Q0.copy(order="F")
    O.Oracle(cfg).advance(Qo, steps)
    s = _solver(cfg.replace(precision="fp32"))
    q, q1 = s.from_numpy(Q0), s.new_state()
    s.advance(q, q1, steps)
    err = rel_l2(s.to_numpy(q), Qo)
    assert err < FP32_TOL, f"{name}: rel L2 {err:.3e}"


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_tile_matches_separate_kernels(prec):
    cfg = config.fh_box(16, precision=prec, seed=3)
    Q0 = ic.equilibrium(cfg)
    out = {}
    for tile in (1, 0):
        s = _solver(cfg, tile)
        q, q1 = s.from_numpy(Q0), s.new_state()
        s.advance(q, q1, 20)
        out[tile] = s.to_numpy(q)
        s.close()
    tol = 1e-13 if prec == "fp64" else 1e-6
    assert rel_l2(out[1], out[0]) < tol


def test_tile_ensemble_equals_boxes_alone():
    from hermeshd_gb300.solver import Ensemble, Solver
    base = config.fh_box(8, precision="fp32", seed=0)
    dx = base.lx / 8
    dims = [(16, 16, 16), (8, 8, 8), (24, 16, 8), (12, 10, 6)]
    seeds = [11, 12, 13, 14]
    ens = Ensemble(base, dims, [(d[0] * dx, d[1] * dx, d[2] * dx) for d in dims], seeds=seeds)
    ens.set_launch(tile_stage=1)
    q, q1 = ens.new_state(), ens.new_state()
    for i in range(ens.nbox):
        v = ens.box_view(q, i)
        v[0, 0].fill_(1.0)
        v[0, 4].fill_(1.0 / (base.aindex - 1.0))
    ens.advance(q, q1, 6)
    for i, (d, sd) in enumerate(zip(dims, seeds)):
        c = base.replace(nx=d[0], ny=d[1], nz=d[2], lx=d[0] * dx, ly=d[1] * dx, lz=d[2] * dx, seed=sd)
        s = Solver(c)
        s.set_launch(tile_stage=1)
        qs, qs1 = s.new_state(), s.new_state()
        qs[0, 0].fill_(1.0)
        qs[0, 4].fill_(1.0 / (base.aindex - 1.0))
        s.advance(qs, qs1, 6)
        assert bool((qs == ens.box_view(q, i)).all()), f"box {i}"
        s.close()
    ens.close()


def test_tile_graph_steps_bit_identical():
    cfg = config.taylor_green_3d(n=16, precision="fp32")
    Q0 = ic.taylor_green(cfg, perturb=1e-3, seed=2)
    res = []
    for k in (1, 4):
        s = _solver(cfg)
        s.set_launch(tile_stage=1, steps_per_graph=k)
        q, q1 = s.from_numpy(Q0), s.new_state()
        s.advance(q, q1, 8)
        res.append(s.to_numpy(q))
        s.close()
    assert np.array_equal(res[0], res[1])

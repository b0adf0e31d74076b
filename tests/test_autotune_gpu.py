"""Launch shapes and the autotuner: every launch shape gives the same result
bit for bit, bad shapes are rejected, and tuning leaves the context where a
fresh one would start (time and stochastic-stress step counter)."""
import numpy as np
import pytest

from hermeshd_gb300 import config, ic

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def test_launch_defaults_and_validation():
    from hermeshd_gb300._lib import HermesError
    from hermeshd_gb300.solver import Solver
    s = Solver(config.sod_1d(nx=64))
    assert s.get_launch() == {"face_tpb": 128, "dt_tpb": 256, "steps_per_graph": 1, "noise_inline": 0,
                              "face_traces": 0, "split_update": 1, "tile_stage": 0, "pdl": 0, "faces_merged": 1,
                              "update_tpb": 128, "cell_concurrent": 1}   # 1-D: no fused stage by default
    for bad in ({"face_tpb": 96}, {"face_tpb": 256}, {"dt_tpb": 48}, {"dt_tpb": 512}, {"steps_per_graph": 65},
                {"update_tpb": 32}, {"update_tpb": 512}):
        with pytest.raises(HermesError):
            s.set_launch(**bad)
    s.set_launch(face_tpb=32, dt_tpb=64, steps_per_graph=4, update_tpb=256)
    assert s.get_launch() == {"face_tpb": 32, "dt_tpb": 64, "steps_per_graph": 4, "noise_inline": 0,
                              "face_traces": 0, "split_update": 1, "tile_stage": 0, "pdl": 0, "faces_merged": 1,
                              "update_tpb": 256, "cell_concurrent": 1}
    with pytest.raises(HermesError):   # no trace kernel for nbasis 4
        s.set_launch(face_traces=1)
    s.set_launch(tile_stage=1)          # the fused stage exists for nbasis 4 and may be forced on
    assert s.get_launch()["tile_stage"] == 1
    s10 = Solver(config.isentropic_vortex_2d(n=8))
    with pytest.raises(HermesError):   # no fused stage for nbasis 10
        s10.set_launch(tile_stage=1)
    s4 = Solver(config.fh_box(8, precision="fp32"))
    assert s4.get_launch()["tile_stage"] == 0   # off by default, available for nbasis 4
    assert s4.get_launch()["faces_merged"] == 0   # FP32 nb 4 below 2^15 cells: a thread per face point
    assert Solver(config.fh_box(32, precision="fp32")).get_launch()["faces_merged"] == 2   # the point loop
    assert s4.get_launch()["update_tpb"] == 64   # FP32 default; 0 selects it again
    s4.set_launch(update_tpb=256)
    assert s4.get_launch()["update_tpb"] == 256
    s4.set_launch()
    assert s4.get_launch()["update_tpb"] == 64
    s4.set_launch(tile_stage=1)
    assert s4.get_launch()["tile_stage"] == 1


@pytest.mark.parametrize("mk", [lambda: config.isentropic_vortex_2d(n=12),
                                lambda: config.fh_box(6, precision="fp32", seed=3)])
def test_every_launch_shape_is_bit_identical(mk):
    from hermeshd_gb300.solver import Solver
    cfg = mk()
    Q = ic.isentropic_vortex(cfg) if cfg.nbasis == 10 else ic.equilibrium(cfg)
    ref = None
    shapes = [{}, {"face_tpb": 32, "dt_tpb": 64, "steps_per_graph": 3},
              {"face_tpb": 64, "dt_tpb": 128, "steps_per_graph": 2, "pdl": 1},
              {"faces_merged": 0}, {"faces_merged": 1}, {"faces_merged": 2},
              {"faces_merged": 2, "noise_inline": 1}, {"update_tpb": 64}, {"update_tpb": 256},
              {"cell_concurrent": 0}, {"cell_concurrent": 0, "steps_per_graph": 3, "faces_merged": 0}]
    if cfg.ivis < 2 and (cfg.precision == "fp32" or not cfg.llns):   # the cell update in one kernel
        shapes.append({"split_update": 0})
    if cfg.llns:   # the stochastic stress drawn inside the face and cell kernels instead of staged
        shapes.append({"noise_inline": 1})
    for shape in shapes:
        s = Solver(cfg)
        # the separate kernels' launch shapes (the fused stage, on by default
        # for this box, has its own bit-identity tests in test_tile_gpu.py)
        s.set_launch(**dict(shape, tile_stage=0) if s.get_launch()["tile_stage"] else shape)
        q, q1 = s.from_numpy(Q), s.new_state()
        t, dt = s.advance(q, q1, 7)
        out = (s.to_numpy(q), t, dt)
        if ref is None:
            ref = out
        else:
            assert np.array_equal(out[0], ref[0]) and out[1] == ref[1] and out[2] == ref[2], shape


def test_face_traces_match_face_evaluation():
    """The trace kernel's values (mirror-pair sums) against the face kernels'
    own evaluation: the same right-hand side to rounding, and 7 steps apart by
    rounding only; with traces off the launch shapes stay bit-identical."""
    from hermeshd_gb300.solver import Solver
    cfg = config.isentropic_vortex_2d(n=12)
    Q = ic.isentropic_vortex(cfg)
    out = {}
    for ft in (1, 0):
        s = Solver(cfg)
        assert s.get_launch()["face_traces"] == 1
        s.set_launch(face_traces=ft)
        assert s.get_launch()["face_traces"] == ft
        q, q1 = s.from_numpy(Q), s.new_state()
        r = s.rhs(q, limit=False)
        s.advance(q, q1, 7)
        out[ft] = (r, q)
    torch = _torch()
    rel = lambda a, b: float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
    assert rel(out[1][0], out[0][0]) < 1e-14
    assert rel(out[1][1], out[0][1]) < 1e-13


def test_autotune_resets_state_and_caches(tmp_path, monkeypatch):
    from hermeshd_gb300 import autotune
    from hermeshd_gb300.solver import Ensemble
    monkeypatch.setenv("HERMES_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    base = config.fh_box(8, precision="fp32", seed=0)
    dims = [(8, 8, 8), (6, 6, 6), (10, 10, 10)]
    dx = base.lx / 8
    lengths = [(n * dx,) * 3 for (n, _, _) in dims]
    ens = Ensemble(base, dims, lengths, seeds=[0, 1, 2])
    q = ens.new_state()
    for i in range(ens.nbox):
        v = ens.box_view(q, i)
        v[0, 0].fill_(1.0)
        v[0, 4].fill_(1.0 / (base.aindex - 1.0))
    r = autotune.autotune(ens, q, steps=2, repeats=2)
    assert not r["cached"] and r["ms_per_step"] <= r["default_ms_per_step"]
    assert set(r["launch"]) == {"face_tpb", "dt_tpb", "steps_per_graph", "noise_inline", "face_traces",
                                "split_update", "tile_stage", "pdl", "faces_merged", "update_tpb",
                                "cell_concurrent"}
    assert ens.get_launch() == r["launch"]
    # tuning stepped copies of q; the context's time and noise counter are reset
    qa, qa1 = q.clone(), ens.new_state()
    ens.advance(qa, qa1, 5)
    fresh = Ensemble(base, dims, lengths, seeds=[0, 1, 2])
    fresh.set_launch(**r["launch"])   # the fused stage and the separate kernels agree to rounding only
    qb, qb1 = q.clone(), fresh.new_state()
    fresh.advance(qb, qb1, 5)
    assert _torch().equal(qa, qb)
    r2 = autotune.autotune(fresh, q, steps=2, repeats=2)
    assert r2["cached"] and r2["launch"] == r["launch"]

"""The autotuner's coordinate search on the CPU, with a stand-in solver whose
step time is a known function of the launch shape: the knobs it tries for a
context (only those the context has), the order it tries them in, and that it
applies and reports the fastest shape and resets the time and noise counter."""
import types

import pytest

from hermeshd_gb300 import autotune


class FakeSolver:
    def __init__(self, split=1, llns=False, traces=0, tile_ok=False):
        self.cfg = types.SimpleNamespace(llns=llns)
        self.launch = {"face_tpb": 128, "dt_tpb": 256, "steps_per_graph": 1, "noise_inline": 0, "face_traces": traces,
                       "split_update": split, "tile_stage": 0, "pdl": 0, "faces_merged": 1, "update_tpb": 128,
                       "cell_concurrent": 1}
        self.tile_ok = tile_ok
        self.calls = []
        self.time = None
        self.step = None

    def get_launch(self):
        return dict(self.launch)

    def set_launch(self, **kw):
        from hermeshd_gb300._lib import HermesError
        new = dict(self.launch)
        new.update({k: v for k, v in kw.items() if v is not None})
        if new["tile_stage"] == 1 and not self.tile_ok:
            raise HermesError(1, "no fused stage")
        self.launch = new
        self.calls.append(dict(new))

    def set_time(self, t):
        self.time = t

    def set_noise_step(self, s):
        self.step = s


class FakeQ:
    def clone(self):
        return self


def cost(launch):
    """ms per step: each knob has one best value."""
    c = 10.0
    c += {128: 0.3, 64: 0.0, 32: 0.2}[launch["face_tpb"]]
    c += {256: 0.1, 128: 0.0, 64: 0.05}[launch["dt_tpb"]]
    c += {1: 0.2, 2: 0.0, 4: 0.1, 8: 0.3}[launch["steps_per_graph"]]
    c += 0.4 if launch["cell_concurrent"] == 0 else 0.0
    c += {64: 0.0, 128: 0.05, 256: 0.1}[launch["update_tpb"]]
    c += {0: 0.2, 1: 0.0, 2: 0.1}[launch["faces_merged"]]
    c += 0.5 * launch["pdl"] + 0.2 * launch["tile_stage"]
    c += 0.0 if launch["split_update"] else 1.0
    c += 0.0 if launch["noise_inline"] else 0.3
    return c


@pytest.fixture
def patched(monkeypatch):
    torch = types.SimpleNamespace(cuda=types.SimpleNamespace(synchronize=lambda: None))
    monkeypatch.setattr(autotune, "_torch", lambda: torch)
    monkeypatch.setattr(autotune, "signature", lambda s: "fake")
    monkeypatch.setattr(autotune, "time_steps", lambda s, q, q1, steps, repeats: cost(s.launch))


def test_search_finds_each_knobs_best_and_applies_it(patched):
    s = FakeSolver(split=1, llns=True)
    r = autotune.autotune(s, FakeQ(), use_cache=False, t0=1.5, step0=7)
    best = {"face_tpb": 64, "dt_tpb": 128, "steps_per_graph": 2, "noise_inline": 1, "split_update": 1, "pdl": 0,
            "faces_merged": 1, "update_tpb": 64, "cell_concurrent": 1}
    for k, v in best.items():
        assert r["launch"][k] == v, (k, r["launch"])
    assert s.launch == r["launch"]
    assert r["ms_per_step"] == pytest.approx(cost(r["launch"]))
    assert r["ms_per_step"] <= r["default_ms_per_step"]
    assert (s.time, s.step) == (1.5, 7)
    assert not r["cached"]


def test_knobs_the_context_lacks_are_not_tried(patched):
    s = FakeSolver(split=0, llns=False, traces=0, tile_ok=False)
    r = autotune.autotune(s, FakeQ(), use_cache=False)
    tuned = set(r["trials"][0]) - {"ms_per_step"}
    assert not tuned & {"noise_inline", "split_update", "update_tpb", "cell_concurrent", "face_traces", "tile_stage"}
    assert {"face_tpb", "dt_tpb", "steps_per_graph", "pdl", "faces_merged"} <= tuned
    # nothing the context lacks was ever set
    assert all(c["tile_stage"] == 0 and c["split_update"] == 0 and c["update_tpb"] == 128 for c in s.calls[1:])
    # the context's current face-kernel variant and concurrency are tried first
    assert r["trials"][0]["faces_merged"] == 1


def test_context_defaults_are_the_first_trial(patched):
    s = FakeSolver(split=1)
    s.launch.update(faces_merged=2, update_tpb=64, cell_concurrent=0)
    r = autotune.autotune(s, FakeQ(), use_cache=False)
    first = r["trials"][0]
    assert (first["faces_merged"], first["update_tpb"], first["cell_concurrent"]) == (2, 64, 0)
    assert r["launch"]["cell_concurrent"] == 1 and r["launch"]["faces_merged"] == 1


def test_cache_returns_the_stored_shape_without_timing(patched, monkeypatch, tmp_path):
    """The first search stores its result under the problem's signature; the
    next call for the same signature applies the stored shape and times
    nothing; a corrupt cache file reads as empty."""
    path = tmp_path / "autotune.json"
    monkeypatch.setenv("HERMES_AUTOTUNE_CACHE", str(path))
    timed = []
    monkeypatch.setattr(autotune, "time_steps", lambda s, q, q1, steps, repeats: timed.append(1) or cost(s.launch))
    s = FakeSolver()
    r1 = autotune.autotune(s, FakeQ(), use_cache=True)
    assert not r1["cached"] and path.exists() and len(timed) > 1
    n = len(timed)
    s2 = FakeSolver()
    r2 = autotune.autotune(s2, FakeQ(), use_cache=True)
    assert r2["cached"] and len(timed) == n
    assert s2.launch == r1["launch"] and r2["ms_per_step"] == r1["ms_per_step"]
    path.write_text("{not json")
    r3 = autotune.autotune(FakeSolver(), FakeQ(), use_cache=True)
    assert not r3["cached"] and len(timed) > n

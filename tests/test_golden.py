"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py
from the FP64 oracle): the oracle must keep reproducing them, and the CUDA
path must match them without the oracle at run time.

Tolerances (relative L2): oracle vs fixture 1e-13 (libm differences between
hosts in the noise path's log/cos); CUDA path: right-hand side 1e-12, state
after the fixture's steps 1e-11, time 1e-11.  The second, numpy restatement
of the step (test_oracle_*_restatement.py) reproduces every fixture,
the stochastic stress and the body force included: measured right-hand sides
within 6e-14, states within 6e-16 (Sod with HLLC 3.6e-13, its contact
branches picked by rounding-level velocities), times within 1e-16.
"""
import glob
import json
import os

import numpy as np
import pytest

from hermeshd_gb300 import config
from helpers import rel_l2

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(HERE, "*.npz")))


def load(name):
    d = np.load(os.path.join(HERE, name + ".npz"))
    cfg = config.Config(**json.loads(str(d["config"])))
    return cfg, {k: d[k] for k in d.files if k != "config"}


def test_fixtures_present():
    assert len(FIXTURES) >= 9


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_reproduces_fixture(name):
    import oracle as O
    cfg, d = load(name)
    o = O.Oracle(cfg)
    Q0 = np.asfortranarray(d["Q0"])
    assert rel_l2(o.rhs(Q0.copy(order="F"), limit=True), d["rhs"]) <= 1e-13
    Q = Q0.copy(order="F")
    t, dt = o.advance(Q, int(d["steps"]))
    assert rel_l2(Q, d["Q"]) <= 1e-13
    assert t == pytest.approx(float(d["t"]), rel=1e-13)


@pytest.mark.gpu
@pytest.mark.parametrize("name", FIXTURES)
def test_cuda_path_matches_fixture(name):
    from hermeshd_gb300.solver import Solver
    cfg, d = load(name)
    s = Solver(cfg)
    q = s.from_numpy(d["Q0"])
    r = s.rhs(q.clone(), limit=True)
    assert rel_l2(s.to_numpy(r), d["rhs"]) <= 1e-12
    q1 = s.new_state()
    t, dt = s.advance(q, q1, int(d["steps"]), t=0.0)
    assert rel_l2(s.to_numpy(q), d["Q"]) <= 1e-11
    assert t == pytest.approx(float(d["t"]), rel=1e-11)


# the numpy restatement of the step reproduces every fixture without the C
# oracle that wrote them -- the right-hand side to 1e-13, the states after the
# fixture's steps to 1e-11 (the two sum in different orders, and the Sod shock
# amplifies those roundings to ~4e-13 in 20 steps)
@pytest.mark.parametrize("name", FIXTURES)
def test_second_restatement_reproduces_fixture(name):
    from test_limiter_restatement import limiter_numpy
    from test_oracle_rhs_restatement import restated_rhs
    from test_oracle_step_restatement import face_basis, step
    cfg, d = load(name)
    B = face_basis(cfg)
    Q0 = np.asfortranarray(d["Q0"])
    assert rel_l2(restated_rhs(cfg, limiter_numpy(Q0, cfg, B)), d["rhs"]) <= 1e-13
    Q, t = Q0.copy(), 0.0
    for n in range(int(d["steps"])):
        Q, dt = step(cfg, Q, B, n)
        t += dt
    assert rel_l2(Q, d["Q"]) <= 1e-11
    assert t == pytest.approx(float(d["t"]), rel=1e-13)

"""The oracle against outputs of the reference's OWN routines: the fixtures
in tests/golden/reference/ were made by tests/golden/make_reference_vectors.py,
which executes the reference's Fortran source (initialize.f90,
basis_funcs.f90, flux.f90 and the 10-moment Roe routine) statement by
statement through tests/golden/fortran_subset.py, no compiler for it being
available.  The basis tables must agree bit for bit, the limiter and the
face fluxes to rounding."""
import os

import numpy as np
import pytest

from hermeshd_gb300 import config

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference")
NBQ = {4: 2, 8: 2, 10: 3}


def load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


@pytest.mark.parametrize("nb", [4, 8, 10])
def test_tables_are_the_references(nb):
    """set_internal_vals_3D, set_face_vals_3D, set_weights_3D,
    set_cbasis_3D and init_bf_weights as the reference runs them."""
    import oracle as O
    iq = NBQ[nb]
    T = load(f"tables_nb{nb}")
    o = O.Oracle(config.Config(nx=2, ny=2, nz=2, nbasis=nb, iquad=iq))
    for ref, orc in (("bfvals_int", "int"), ("bfvals_xp", "xp"), ("bfvals_xm", "xm"), ("bfvals_yp", "yp"),
                     ("bfvals_ym", "ym"), ("bfvals_zp", "zp"), ("bfvals_zm", "zm")):
        assert np.array_equal(o.table(orc)[:, :nb], T[ref]), ref
    assert np.array_equal(o.table("faces")[:6 * iq * iq, :nb], T["bf_faces"][:6 * iq * iq])
    assert np.array_equal(o.table("cbasis")[:nb], T["cbasis"])
    assert np.array_equal(o.table("wgt3d")[:iq ** 3], T["wgt3d"])
    assert np.array_equal(o.table("wgt2d")[:iq * iq], T["wgt2d"])


@pytest.mark.parametrize("nb", [4, 8, 10])
def test_limiter_is_the_references(nb):
    import oracle as O
    d = load(f"limiter_nb{nb}")
    before = np.asfortranarray(d["before"])
    nx, ny, nz = before.shape[:3]
    cfg = config.Config(nx=nx, ny=ny, nz=nz, nbasis=nb, iquad=NBQ[nb], rh_floor=float(d["rh_floor"]),
                        T_floor=float(d["T_floor"]), aindex=float(d["aindex"]))
    got = before.copy(order="F")
    O.Oracle(cfg).limiter(got)
    assert not np.array_equal(d["after"], before)                    # the reference's limiter acted
    assert np.allclose(got, d["after"], rtol=1e-13, atol=1e-15), float(np.abs(got - d["after"]).max())


def test_face_fluxes_are_the_references():
    """Piecewise-constant three-cell periodic lines: the oracle's cell-average
    right-hand side is dxi (F(q_i, q_i+1) - F(q_i-1, q_i)) with F the
    reference's face flux (coll 0: no sources)."""
    import oracle as O
    d = load("faces")
    n = len(d["dir"])
    assert n >= 50
    for r in range(n):
        ax = int(d["dir"][r]) - 1
        dims, lens = [1, 1, 1], [0.5, 0.5, 0.5]
        dims[ax], lens[ax] = 3, 1.5
        cfg = config.Config(nx=dims[0], ny=dims[1], nz=dims[2], lx=lens[0], ly=lens[1], lz=lens[2], nbasis=4,
                            iquad=2, iorder=2, ivis=int(d["ivis"][r]), ieos=int(d["ieos"][r]),
                            ihllc=int(d["solver"][r]), coll=0.0, colvis=float(d["colvis"]),
                            aindex=float(d["aindex"]), P_1=float(d["P_1"]), P_base=float(d["P_base"]),
                            rh_floor=float(d["rh_floor"]), T_floor=float(d["T_floor"]))
        Q = np.zeros(cfg.shape_f, order="F")
        for i in range(3):
            idx = [0, 0, 0]
            idx[ax] = i
            Q[idx[0], idx[1], idx[2], :, 0] = d["states"][r][i]
        got = O.Oracle(cfg).rhs(Q, limit=False)
        F = d["fluxes"][r]
        for i in range(3):
            idx = [0, 0, 0]
            idx[ax] = i
            want = 2.0 * (F[i] - F[(i - 1) % 3])                      # dxi = 3 / 1.5
            row = got[idx[0], idx[1], idx[2], :, 0]
            assert np.allclose(row, want, rtol=1e-12, atol=1e-13 * np.abs(want).max()), (r, i, row - want)


STEPS = sorted(os.path.splitext(f)[0][len("step_"):] for f in os.listdir(HERE) if f.startswith("step_"))
TWINS = [n for n in STEPS if os.path.exists(os.path.join(os.path.dirname(HERE), n + ".npz"))]


def load_step(name):
    import json
    d = load("step_" + name)
    return config.Config(**json.loads(str(d["config"]))), d


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


def test_step_fixtures_present():
    assert len(STEPS) >= 6


@pytest.mark.parametrize("name", STEPS)
def test_oracle_reproduces_the_references_step(name):
    """The reference's whole step, executed from its source: the oracle's
    right-hand side (limiter applied) and its state and time after the
    fixture's steps (measured: identical for Sod, walls and Taylor-Green,
    within 1e-15 for the nb-10 vortex)."""
    import oracle as O
    cfg, d = load_step(name)
    o = O.Oracle(cfg)
    Q0 = np.asfortranarray(d["Q0"])
    assert rel_l2(o.rhs(Q0.copy(order="F"), limit=True), d["rhs"]) <= 1e-13
    Q = Q0.copy(order="F")
    t, dt = o.advance(Q, int(d["steps"]))
    assert rel_l2(Q, d["Q"]) <= 1e-13
    assert t == pytest.approx(float(d["t"]), rel=1e-14)


@pytest.mark.parametrize("name", TWINS)
def test_oracle_written_fixture_is_the_references(name):
    """The golden fixture of the same name, written by the oracle and read by
    the CUDA path's fixture test, equals the reference-executed one: that
    test holds the GPU to the reference's own outputs."""
    g = dict(np.load(os.path.join(os.path.dirname(HERE), name + ".npz")))
    _, d = load_step(name)
    assert np.array_equal(g["Q0"], d["Q0"])
    assert rel_l2(g["rhs"], d["rhs"]) <= 1e-13
    assert rel_l2(g["Q"], d["Q"]) <= 1e-13
    assert float(g["t"]) == pytest.approx(float(d["t"]), rel=1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("name", TWINS)
def test_cuda_path_matches_the_references_step(name):
    """The CUDA path against the reference's executed step, on the cases whose
    oracle-written twins the CUDA path's fixture test already reads (the
    other cases are held to the oracle bit for bit above)."""
    from hermeshd_gb300.solver import Solver
    cfg, d = load_step(name)
    s = Solver(cfg)
    q = s.from_numpy(d["Q0"])
    r = s.rhs(q.clone(), limit=True)
    assert rel_l2(s.to_numpy(r), d["rhs"]) <= 1e-12
    q1 = s.new_state()
    t, dt = s.advance(q, q1, int(d["steps"]), t=0.0)
    assert rel_l2(s.to_numpy(q), d["Q"]) <= 1e-11
    assert t == pytest.approx(float(d["t"]), rel=1e-11)


def test_ivis2_stage_writes_only_the_stresses():
    """The reference's own ivis-2 stage (integrator.f90:181-228), run into an
    output prefilled with 7.0, leaves rh..en unwritten -- the deviation the
    oracle and the CUDA path state (they give those rows the explicit
    update) -- and its stress rows are the oracle's bit for bit."""
    import json
    import oracle as O
    d = load("ivis2_stage")
    cfg = config.Config(**json.loads(str(d["config"])))
    assert np.all(d["Q_out"][..., :5, :] == 7.0)
    e = O.Oracle(cfg).euler_step(np.asfortranarray(d["Q_in"]).copy(order="F"), float(d["dt"]))
    assert np.array_equal(e[..., 5:, :], d["Q_out"][..., 5:, :])


def test_grad_closure_faces_are_the_monoliths():
    """ivis 3 face fluxes against the Grad-closure monolith's own point flux,
    freezing speed and HLLC (dg_3D_hydro_bitri_ten_moment.f90), executed."""
    import oracle as O
    d = load("faces_grad")
    assert len(d["dir"]) >= 12
    for r in range(len(d["dir"])):
        ax = int(d["dir"][r]) - 1
        dims, lens = [1, 1, 1], [0.5, 0.5, 0.5]
        dims[ax], lens[ax] = 3, 1.5
        cfg = config.Config(nx=dims[0], ny=dims[1], nz=dims[2], lx=lens[0], ly=lens[1], lz=lens[2], nbasis=4,
                            iquad=2, iorder=2, ivis=3, ihllc=int(d["solver"][r]), coll=0.0, colvis=0.0,
                            aindex=float(d["aindex"]), rh_floor=float(d["rh_floor"]), T_floor=float(d["T_floor"]))
        Q = np.zeros(cfg.shape_f, order="F")
        for i in range(3):
            idx = [0, 0, 0]
            idx[ax] = i
            Q[idx[0], idx[1], idx[2], :, 0] = d["states"][r][i]
        got = O.Oracle(cfg).rhs(Q, limit=False)
        F = d["fluxes"][r]
        for i in range(3):
            idx = [0, 0, 0]
            idx[ax] = i
            want = 2.0 * (F[i] - F[(i - 1) % 3])
            assert np.allclose(got[idx[0], idx[1], idx[2], :, 0], want, rtol=1e-12, atol=1e-13 * np.abs(want).max())


def test_grad_closure_source_step_reading():
    """The monolith's implicit source step run on the same advected state:
    with distinct input and output it is the oracle's RK2 stage bit for bit
    (the order-independent reading the oracle and the CUDA path take); as the
    monolith calls it, with one array as both (each update reading the ones
    before it), it differs from that by ~3e-6 of the stresses per stage --
    the size of the choice between the two readings of that call."""
    import json
    import oracle as O
    d = load("grad_source_step")
    cfg = config.Config(**json.loads(str(d["config"])))
    e = O.Oracle(cfg).euler_step(np.asfortranarray(d["Q"]).copy(order="F"), float(d["dt"]))
    assert np.array_equal(e, d["separate"])
    gap = np.abs(e - d["aliased"]).max() / np.abs(e).max()
    assert 1e-8 < gap < 1e-4, gap


@pytest.mark.parametrize("icid", [1, 2, 3, 4, 5])
def test_initial_states_are_the_references(icid):
    """set_ic (initialcon.f90:20-72) executed for the isentropic vortex v0/v1,
    the Sod tube v0/v1 and the Poiseuille fluid at rest: the host
    restatement ic.from_icid, which the device initial states are tested
    against, reproduces it to one rounding."""
    import json
    from hermeshd_gb300 import ic
    d = load("initial_states")
    cfg = config.Config(**json.loads(str(d[f"config_{icid}"])))
    ref = d[f"Q_{icid}"]
    assert np.allclose(ic.from_icid(cfg, icid), ref, rtol=0, atol=4e-16 * np.abs(ref).max())

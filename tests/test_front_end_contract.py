"""The reference-facing front end (hermeshd.Hermeshd) takes host field arrays
as the f2py extension does (intent(inout), src/hermeshd.py:46): used as given
or rejected, never converted.  The reference driver passes float32
Fortran-ordered arrays (src/test_hermeshd.py:48-50, nx 50, nbasis 8), which
run on the FP32 path; float64 arrays run on the FP64 path.

The rejections happen before a context exists, so they run without a GPU;
the reference script's loop itself is a GPU test."""
import numpy as np
import pytest

from hermeshd_gb300 import config, ic
from hermeshd_gb300._lib import HermesError
from helpers import rel_l2


def _scalars():
    return (np.array(0.0), np.array(0.0), np.array(0.0), np.array(0.0), np.array(0.0), np.array(0))


def _module(cfg):
    from hermeshd_gb300 import hermeshd as H
    m = H.Hermeshd()
    m.configure(cfg, icid=3)
    return m


@pytest.mark.parametrize("prec,wrong", [("fp64", np.float32), ("fp32", np.float64)])
def test_dtype_mismatch_is_rejected_not_cast(prec, wrong):
    cfg = config.sod_1d(nx=50, nbasis=8, iquad=2, precision=prec)
    m = _module(cfg)
    Q = np.zeros(cfg.shape_f, order="F", dtype=wrong)
    t, dt, t1, t_start, dtout, nout = _scalars()
    with pytest.raises(HermesError) as e:
        m.setup(Q, t, dt, t1, t_start, dtout, nout, 0)
    assert e.value.code == 3
    with pytest.raises(HermesError) as e:
        m.step(Q, np.zeros_like(Q), np.zeros_like(Q), t, dt)
    assert e.value.code == 3
    assert m.solver is None          # rejected before any device work


def test_shape_and_order_mismatch_are_rejected():
    cfg = config.sod_1d(nx=50, nbasis=8, iquad=2, precision="fp32")
    m = _module(cfg)
    t, dt, *_ = _scalars()
    good = np.zeros(cfg.shape_f, order="F", dtype=np.float32)
    bad_shape = np.zeros((49,) + cfg.shape_f[1:], order="F", dtype=np.float32)
    c_order = np.zeros((50, 1, 1, 11, 8), order="C", dtype=np.float32)
    for q, q1 in ((bad_shape, good), (good, bad_shape), (c_order, good)):
        with pytest.raises(HermesError) as e:
            m.step(q, q1, None, t, dt)
        assert e.value.code == 2
    assert m.solver is None


def test_solver_host_array_layouts():
    """Solver.advance_host takes the two views of the state's memory, a
    C-contiguous (nb,nQ,nz,ny,nx) array or a Fortran-ordered Q(nx,ny,nz,nQ,nb),
    and refuses a C-ordered Q(nx,ny,nz,nQ,nb) of the right size (another
    layout) and the wrong dtype, before any call into the library."""
    from hermeshd_gb300.solver import Solver
    cfg = config.isentropic_vortex_2d(n=6)
    s = Solver.__new__(Solver)            # no context: the checks come first
    s.cfg, s.np_dtype = cfg, np.float64
    for bad, code in ((np.zeros(cfg.shape_f, order="C"), 2),
                      (np.zeros(cfg.shape_c, order="F"), 2),
                      (np.zeros(cfg.shape_c, dtype=np.float32), 3),
                      (np.zeros(cfg.shape_c)[..., ::2], 2)):
        with pytest.raises(HermesError) as e:
            s.advance_host(bad, 1)
        assert e.value.code == code


@pytest.mark.gpu
def test_reference_driver_loop_with_float32_arrays():
    """src/test_hermeshd.py:44-83 as written: float32 Fortran arrays (nx 50,
    nQ 11, nB 8), 0-d float64 scalars mutated in place, setup / step /
    generate_output until t >= tf = 7e-4 (one CFL step of this grid), then 9
    more steps through the same calls, cleanup.  The FP32 state is held
    against the FP64 oracle over the same steps (FP32 bound 1e-5)."""
    import oracle as O
    cfg = config.sod_1d(nx=50, nbasis=8, iquad=2, precision="fp32")
    m = _module(cfg)
    Qio = np.empty(cfg.shape_f, order="F", dtype=np.float32)
    Q1 = np.empty(cfg.shape_f, order="F", dtype=np.float32)
    Q2 = np.empty(cfg.shape_f, order="F", dtype=np.float32)
    t, tf, dt = np.array(0.0), np.array(7.0e-4), np.array(0.0)
    t1, t_start, dtout, nout = np.array(0.0), np.array(0.0), np.array(0.0), np.array(0)
    m.setup(Qio, t, dt, t1, t_start, dtout, nout, 0)
    assert Qio.dtype == np.float32
    o = O.Oracle(cfg.replace(precision="fp64"))
    Qo = ic.sod(cfg)
    to, n = 0.0, 0

    def one():
        nonlocal to, n
        m.step(Qio, Q1, Q2, t, dt)
        m.generate_output(Qio, t, dt, t1, dtout, nout)
        to, _ = o.step(Qo, o.new(), o.new(), to, 0.0)
        n += 1

    while t < tf:
        one()
    assert n >= 1 and float(t) >= 7.0e-4
    for _ in range(9):
        one()
    m.cleanup(t_start)
    assert Qio.dtype == np.float32 and Q1.dtype == np.float32
    assert abs(float(t) - to) <= 1e-5 * to
    assert rel_l2(Qio, Qo) < 1e-5

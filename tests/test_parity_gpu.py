"""GPU parity: the CUDA path (through the C ABI) against the FP64 oracle.

Tolerances (relative L2 over the whole field array):
  one right-hand side / one limiter pass     1e-12
  100 steps of the FP64 step                 1e-11   (the stated FP64 bar)
  FP32 path vs the FP64 oracle               1e-5
"""
import numpy as np
import pytest

from hermeshd_gb300 import config, ic
from helpers import rel_l2

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
STEP_TOL = 1e-11
FP32_TOL = 1e-5


def _solver(cfg):
    from hermeshd_gb300.solver import Solver
    return Solver(cfg)


def _oracle(cfg):
    import oracle as O
    return O.Oracle(cfg)


RHS_CASES = {
    "nb4_3d_periodic_ivis0": (config.Config(nx=6, ny=5, nz=4, nbasis=4, iquad=2, ivis=0, coll=0.7, lx=1.3, ly=0.9, lz=1.1), 2.0),
    "nb8_2d_wall_ivis1": (config.Config(nx=8, ny=7, nz=1, nbasis=8, iquad=2, ivis=1, coll=3.0, colvis=1.5,
                                        xlobc="wall", xhibc="wall", ly=0.8), 1.0),
    "nb10_2d_periodic": (config.Config(nx=6, ny=6, nz=1, nbasis=10, iquad=3, ivis=0, aindex=1.4), 0.0),
    "nb10_3d_mixed_bc": (config.Config(nx=5, ny=4, nz=3, nbasis=10, iquad=3, ivis=1, coll=2.0, colvis=1.0,
                                       xlobc="outflow", xhibc="wall", ylobc="noslip", yhibc="outflow",
                                       zlobc="wall", zhibc="noslip"), 0.5),
    "nb4_3d_ivis2": (config.Config(nx=5, ny=4, nz=3, nbasis=4, iquad=2, ivis=2, coll=1.5, colvis=1.0), 1.0),
    "nb8_3d_ivis2_walls": (config.Config(nx=4, ny=5, nz=3, nbasis=8, iquad=2, ivis=2, coll=1.5, colvis=1.0,
                                         ylobc="wall", yhibc="noslip"), 1.0),
    "nb8_3d_noise": (config.Config(nx=4, ny=4, nz=4, nbasis=8, iquad=2, ivis=1, coll=1.0, colvis=1.0, llns=True,
                                   eta_sd=0.05, zeta_sd=0.01, seed=1234), 0.5),
    "nb4_2d_bodyforce_noslip": (config.Config(nx=6, ny=8, nz=1, nbasis=4, iquad=2, ivis=1, coll=5.0, colvis=1.0,
                                              ylobc="noslip", yhibc="noslip", body_force=0.1), 0.0),
    "nb4_x_periodic_hi_only": (config.Config(nx=6, ny=3, nz=2, nbasis=4, iquad=2, xlobc="wall", xhibc="periodic"), 0.0),
    # Roe solver of the monolithic code (ihllc = 2)
    "nb4_3d_roe": (config.Config(nx=5, ny=4, nz=3, nbasis=4, iquad=2, ihllc=2), 0.0),
    "nb10_2d_roe_walls_ivis1": (config.Config(nx=6, ny=5, nz=1, nbasis=10, iquad=3, ihllc=2, ivis=1, coll=2.0,
                                              colvis=1.0, xlobc="wall", xhibc="wall"), 0.5),
    "nb8_3d_central_only": (config.Config(nx=4, ny=4, nz=3, nbasis=8, iquad=2, ihllc=0), 0.0),
    # degenerate extents: one cell across a direction, a single cell
    "nb8_one_cell_x": (config.Config(nx=1, ny=5, nz=3, nbasis=8, iquad=2, ivis=1, coll=2.0, colvis=1.0), 0.5),
    "nb4_line_walls": (config.Config(nx=7, ny=1, nz=1, nbasis=4, iquad=2, xlobc="wall", xhibc="noslip"), 0.0),
    "nb10_single_cell": (config.Config(nx=1, ny=1, nz=1, nbasis=10, iquad=3), 0.0),
    # Murnaghan-Tait equation of state (ieos 2), with the HLLC sound speed's stale 1/rho (flux.f90:533-534)
    "nb4_2d_tait_hllc_walls": (config.Config(nx=6, ny=5, nz=1, nbasis=4, iquad=2, ieos=2, P_1=0.05, P_base=1.0,
                                             xlobc="wall", xhibc="noslip"), 0.0),
    "nb10_2d_tait_roe": (config.Config(nx=5, ny=5, nz=1, nbasis=10, iquad=3, ieos=2, P_1=0.05, P_base=1.0,
                                       ihllc=2), 0.0),
    # parabolic x-low inflow (boundary.f90:568-612)
    "nb4_2d_inflow_noslip": (config.Config(nx=6, ny=8, nz=1, nbasis=4, iquad=2, ivis=1, coll=3.0, colvis=1.0,
                                           xlobc="inflow", xhibc="wall", ylobc="noslip", yhibc="noslip",
                                           inflow_u=0.3, inflow_p=1.0), 0.5),
    "nb10_2d_inflow_roe": (config.Config(nx=5, ny=6, nz=1, nbasis=10, iquad=3, ihllc=2, xlobc="inflow",
                                         xhibc="noslip", ylobc="wall", yhibc="wall", inflow_u=0.5,
                                         inflow_rho=1.2, inflow_p=0.8), 0.0),
    # Grad closure (ivis 3, E_ij form)
    "nb4_3d_grad": (config.Config(nx=5, ny=4, nz=3, nbasis=4, iquad=2, ivis=3, coll=1.5), 1.0),
    "nb10_2d_grad_roe": (config.Config(nx=5, ny=6, nz=1, nbasis=10, iquad=3, ivis=3, coll=0.5, ihllc=2), 1.0),
}


@pytest.mark.parametrize("name", sorted(RHS_CASES))
def test_rhs_parity(name):
    cfg, stress = RHS_CASES[name]
    Q = ic.random_smooth(cfg, seed=7, amp=0.1, stress_amp=0.05 * stress)
    if cfg.ivis >= 2:
        Q = ic.ten_moment_stress(cfg, Q, p=1.0, amp=0.01)
    o = _oracle(cfg)
    Qo = Q.copy(order="F")
    r_o = o.rhs(Qo, limit=True)
    s = _solver(cfg)
    q = s.from_numpy(Q)
    r_g = s.to_numpy(s.rhs(q, limit=True))
    # the limiter writes q in place on both sides
    assert rel_l2(s.to_numpy(q), Qo) < RHS_TOL
    err = rel_l2(r_g, r_o)
    assert err < RHS_TOL, f"{name}: rel L2 {err:.3e}"


def test_limiter_active_parity():
    """A state whose face densities and pressures dip below the floors, so
    every limiter branch runs (flux.f90:1077-1164)."""
    cfg = config.Config(nx=16, ny=8, nz=2, nbasis=8, iquad=2, T_floor=2.0)
    rng = np.random.default_rng(3)
    Q = ic.random_smooth(cfg, seed=11, amp=0.2)
    sh = (cfg.nx, cfg.ny, cfg.nz)
    Q[:, :, :, 0, 1:] = 0.6 * rng.standard_normal(sh + (cfg.nbasis - 1,))   # big density slopes
    Q[:, :, :, 4, 1:] = 1.5 * rng.standard_normal(sh + (cfg.nbasis - 1,))
    Q[::5, :, :, 0, 0] = 1e-7                                                # below rh_floor
    o = _oracle(cfg)
    Qo = Q.copy(order="F")
    o.limiter(Qo)
    s = _solver(cfg)
    q = s.from_numpy(Q)
    s.limiter(q)
    g = s.to_numpy(q)
    assert not np.array_equal(Qo, Q)   # the limiter did something
    assert rel_l2(g, Qo) < RHS_TOL


def test_min_dt_parity():
    cfg = config.isentropic_vortex_2d(n=16)
    Q = ic.isentropic_vortex(cfg)
    o = _oracle(cfg)
    s = _solver(cfg)
    dt_o = o.get_min_dt(Q.copy(order="F"))
    dt_g = s.get_min_dt(s.from_numpy(Q))
    assert abs(dt_g - dt_o) <= 1e-14 * dt_o


STEP_CASES = {
    "sod_256_rk2_nb4": (lambda: config.sod_1d(nx=256), lambda c: ic.sod(c)),
    "vortex_16_rk3_nb10": (lambda: config.isentropic_vortex_2d(n=16), lambda c: ic.isentropic_vortex(c)),
    # symmetry broken by 1e-3: the exact field sits on the reference HLLC's
    # discontinuity (see ic.taylor_green and test_oracle_kat)
    "tgv_8_rk3_nb4_ivis1": (lambda: config.taylor_green_3d(n=8, precision="fp64"),
                            lambda c: ic.taylor_green(c, perturb=1e-3, seed=1)),
    "random_nb8_walls_rk2": (lambda: config.Config(nx=10, ny=6, nz=3, nbasis=8, iquad=2, ivis=1, coll=2.0, colvis=0.5,
                                                   xlobc="wall", xhibc="noslip", zlobc="outflow", zhibc="wall"),
                             lambda c: ic.random_smooth(c, seed=5, amp=0.05, stress_amp=0.01)),
    "fh_noise_8_rk2_nb4": (lambda: config.fh_box(8, precision="fp64", seed=42), lambda c: ic.equilibrium(c)),
    "sod_256_rk2_roe": (lambda: config.sod_1d(nx=256, ihllc=2), lambda c: ic.sod(c)),
    "grad_rk2_split_source_nb4": (lambda: config.Config(nx=6, ny=5, nz=4, nbasis=4, iquad=2, ivis=3, coll=2.0, iorder=2),
                                  lambda c: ic.ten_moment_stress(c, ic.random_smooth(c, seed=9, amp=0.05), p=1.0, amp=0.01)),
    "tait_rk2_nb4_hllc": (lambda: config.Config(nx=12, ny=10, nz=1, nbasis=4, iquad=2, ieos=2, P_1=0.05, P_base=1.0),
                          lambda c: ic.random_smooth(c, seed=4, amp=0.05)),
    "channel_inflow_rk2_nb4": (lambda: config.Config(nx=16, ny=8, nz=1, lx=2.0, ly=1.0, nbasis=4, iquad=2, ivis=1,
                                                     coll=20.0, colvis=1.0, xlobc="inflow", xhibc="wall",
                                                     ylobc="noslip", yhibc="noslip", inflow_u=0.3, inflow_p=1.0,
                                                     ihllc=2),
                               lambda c: ic.channel(c, amplitude=0.0)),
    "grad_rk3_nb10": (lambda: config.Config(nx=8, ny=8, nz=1, nbasis=10, iquad=3, ivis=3, coll=1.0, iorder=3),
                      lambda c: ic.ten_moment_stress(c, ic.random_smooth(c, seed=2, amp=0.05), p=1.0, amp=0.01)),
}


@pytest.mark.parametrize("name", sorted(STEP_CASES))
def test_100_steps_parity(name):
    mk, icf = STEP_CASES[name]
    cfg = mk()
    Q = icf(cfg)
    o = _oracle(cfg)
    Qo = Q.copy(order="F")
    t_o, dt_o = o.advance(Qo, 100)
    s = _solver(cfg)
    q, q1 = s.from_numpy(Q), s.new_state()
    t_g, dt_g = s.advance(q, q1, 100, t=0.0)
    err = rel_l2(s.to_numpy(q), Qo)
    assert abs(t_g - t_o) <= 1e-11 * t_o
    assert err < STEP_TOL, f"{name}: rel L2 after 100 steps {err:.3e}"


def test_step_equals_graph_advance():
    cfg = config.isentropic_vortex_2d(n=12)
    Q = ic.isentropic_vortex(cfg)
    s = _solver(cfg)
    qa, qa1 = s.from_numpy(Q), s.new_state()
    t = 0.0
    for _ in range(7):
        t, dt = s.step(qa, qa1, None, t)
    qb, qb1 = s.from_numpy(Q), s.new_state()
    tb, dtb = s.advance(qb, qb1, 7, t=0.0)
    assert t == tb and dt == dtb
    assert np.array_equal(s.to_numpy(qa), s.to_numpy(qb))


@pytest.mark.parametrize("case", ["sod_rk2", "vortex_nb10_rk3", "fh_fp32_noise"])
def test_host_buffers_equal_device(case):
    """Host-array stepping equals the device path bit for bit: pageable host
    memory (copied back after the steps) and pinned memory (the last stage
    stores into it directly)."""
    import torch
    cfg = {"sod_rk2": lambda: config.sod_1d(nx=64),
           "vortex_nb10_rk3": lambda: config.isentropic_vortex_2d(n=12),
           "fh_fp32_noise": lambda: config.fh_box(6, precision="fp32", seed=4)}[case]()
    Q = {"sod_rk2": ic.sod, "vortex_nb10_rk3": ic.isentropic_vortex, "fh_fp32_noise": ic.equilibrium}[case](cfg)
    s = _solver(cfg)
    q, q1 = s.from_numpy(Q), s.new_state()
    t_d, _ = s.advance(q, q1, 12)
    ref = s.to_numpy(q).T
    for pinned, conc in ((False, 0), (True, 0), (True, 1)):
        s2 = _solver(cfg)
        s2.set_launch(cell_concurrent=conc)
        qh0 = np.ascontiguousarray(Q.T).astype(s2.np_dtype)   # (nb, nQ, nz, ny, nx) C order = the Fortran memory
        if pinned:
            buf = torch.empty(qh0.shape, dtype=torch.from_numpy(qh0).dtype, pin_memory=True)
            qh = buf.numpy()
            qh[...] = qh0
        else:
            qh = qh0
        t_h, _ = s2.advance_host(qh, 5)
        t_h, _ = s2.advance_host(qh, 7, t=t_h)
        assert t_h == t_d, (pinned, conc, t_h, t_d)
        assert np.array_equal(qh, ref), (pinned, conc)


def test_ensemble_host_buffers_equal_device():
    """An ensemble stepped on a pinned host array (the last stage stores into
    it directly) equals the device path bit for bit."""
    import torch
    from hermeshd_gb300.solver import Ensemble
    base = config.fh_box(6, precision="fp32", seed=0)
    dims = [(6, 6, 6), (4, 5, 3)]
    lengths = [(d[0] * 10.0, d[1] * 10.0, d[2] * 10.0) for d in dims]

    def make():
        e = Ensemble(base, dims, lengths, [5, 6])
        q = e.new_state()
        for i in range(len(dims)):
            v = e.box_view(q, i)
            v.zero_()
            v[0, 0].fill_(1.0)
            v[0, 4].fill_(1.0 / (base.aindex - 1.0))
        return e, q

    e1, q = make()
    e1.advance(q, e1.new_state(), 9)
    e2, q0 = make()
    buf = torch.empty(q0.shape, dtype=q0.dtype, pin_memory=True)
    buf.copy_(q0)
    e2.advance_host(buf.numpy(), 4)
    e2.advance_host(buf.numpy(), 5)
    assert torch.equal(buf, q.cpu())


def test_fp32_path_against_fp64_oracle():
    cfg = config.isentropic_vortex_2d(n=16, precision="fp32")
    Q = ic.isentropic_vortex(cfg)
    o = _oracle(cfg.replace(precision="fp64"))
    Qo = Q.copy(order="F")
    o.advance(Qo, 20)
    s = _solver(cfg)
    q, q1 = s.from_numpy(Q), s.new_state()
    s.advance(q, q1, 20)
    err = rel_l2(s.to_numpy(q), Qo)
    assert err < FP32_TOL, err


def test_nonfinite_is_reported_and_context_survives():
    from hermeshd_gb300._lib import NonFiniteError
    cfg = config.sod_1d(nx=32)
    Q = ic.sod(cfg)
    Qbad = Q.copy(order="F")
    Qbad[5, 0, 0, 4, 0] = np.nan
    s = _solver(cfg)
    q, q1 = s.from_numpy(Qbad), s.new_state()
    with pytest.raises(NonFiniteError):
        s.step(q, q1, None, 0.0)
    # the context and the GPU stay usable
    q, q1 = s.from_numpy(Q), s.new_state()
    t, dt = s.step(q, q1, None, 0.0)
    assert np.isfinite(s.to_numpy(q)).all() and dt > 0
    # host buffers: the non-finite state is copied back and the error raised
    qh = np.ascontiguousarray(Qbad.T)
    with pytest.raises(NonFiniteError):
        s.advance_host(qh, 1)
    assert not np.isfinite(qh).all()
    qh = np.ascontiguousarray(Q.T)
    t, dt = s.advance_host(qh, 2)
    assert np.isfinite(qh).all() and dt > 0


@pytest.mark.parametrize("kind", ["fh_nb4", "nb10_face_traces"])
def test_ensemble_equals_single_boxes(kind):
    """Boxes of uneven sizes stepped as one ensemble == each box alone, bit for
    bit: the fluctuating-hydro box (stochastic stress, per-box Philox key) and
    an FP64 nbasis-10 box, whose face traces go through the grid-wide trace
    buffer (cells of every box in one array)."""
    import torch
    from hermeshd_gb300.solver import Ensemble
    if kind == "fh_nb4":
        base = config.fh_box(8, precision="fp64", seed=0)
        dims = [(8, 8, 8), (6, 6, 6), (4, 5, 3)]
    else:
        base = config.Config(nx=6, ny=5, nz=2, nbasis=10, iquad=3, ivis=1, coll=2.0, colvis=1.0)
        dims = [(6, 5, 2), (4, 4, 3), (5, 3, 1)]
    L = 10.0
    lengths = [(d[0] * L, d[1] * L, d[2] * L) for d in dims]
    seeds = [11, 22, 33]
    ens = Ensemble(base, dims, lengths, seeds)
    q, q1 = ens.new_state(), ens.new_state()
    inits = []
    for i, d in enumerate(dims):
        c = base.replace(nx=d[0], ny=d[1], nz=d[2], lx=lengths[i][0], ly=lengths[i][1], lz=lengths[i][2], seed=seeds[i])
        Qi = ic.random_smooth(c, seed=i, amp=0.02)
        inits.append((c, Qi))
        ens.box_view(q, i).copy_(torch.from_numpy(np.ascontiguousarray(Qi.T)).to(q.device))
    ens.advance(q, q1, 5)
    t_e, dt_e = ens.box_times()
    for i, (c, Qi) in enumerate(inits):
        s = _solver(c)
        qs, qs1 = s.from_numpy(Qi), s.new_state()
        t_s, dt_s = s.advance(qs, qs1, 5)
        assert t_s == t_e[i]
        assert np.array_equal(s.to_numpy(qs), s.to_numpy(ens.box_view(q, i)))


def test_reference_front_end_step():
    """hermeshd.hermeshd.setup/step with numpy Fortran arrays, as in
    src/test_hermeshd.py:44-78."""
    from hermeshd_gb300 import hermeshd as H
    cfg = config.sod_1d(nx=50)
    mod = H.Hermeshd()
    mod.configure(cfg, icid=3)
    Qio = np.empty(cfg.shape_f, order="F", dtype=np.float64)
    Q1, Q2 = np.empty_like(Qio), np.empty_like(Qio)
    t, dt, t1, t_start, dtout, nout = (np.array(0.0), np.array(0.0), np.array(0.0), np.array(0.0),
                                        np.array(0.0), np.array(0))
    mod.setup(Qio, t, dt, t1, t_start, dtout, nout, 0)
    o = _oracle(cfg)
    Qo = ic.sod(cfg)
    to = 0.0
    for _ in range(5):
        mod.step(Qio, Q1, Q2, t, dt)
        mod.generate_output(Qio, t, dt, t1, dtout, nout)
        to, dto = o.step(Qo, o.new(), o.new(), to, 0.0)
    assert abs(float(t) - to) <= 1e-14 * to
    assert rel_l2(Qio, Qo) < STEP_TOL
    mod.cleanup(t_start)


def test_fh_ensemble_conserves_and_fluctuates():
    """Stochastic stress enters as a face flux: mass and momentum of every box
    are conserved to rounding while density fluctuations develop."""
    import torch
    from hermeshd_gb300.analysis import StructureFactor
    from hermeshd_gb300.solver import Ensemble
    base = config.fh_box(8, precision="fp64", seed=0)
    dx = base.lx / 8
    dims = [(8, 8, 8), (12, 12, 12), (6, 10, 8)]
    ens = Ensemble(base, dims, [(d[0] * dx, d[1] * dx, d[2] * dx) for d in dims], seeds=[3, 4, 5])
    q, q1 = ens.new_state(), ens.new_state()
    for i in range(ens.nbox):
        v = ens.box_view(q, i)
        v[0, 0].fill_(1.0)
        v[0, 4].fill_(1.0 / (base.aindex - 1.0))
    m0 = [float(ens.box_view(q, i)[0, 0].sum()) for i in range(ens.nbox)]
    ens.advance(q, q1, 40)
    sf = StructureFactor(kmax=4)
    for i in range(ens.nbox):
        v = ens.box_view(q, i)
        n = v[0, 0].numel()
        assert abs(float(v[0, 0].sum()) / m0[i] - 1) < 1e-12
        for c in (1, 2, 3):
            assert abs(float(v[0, c].sum())) < 1e-12 * n
        assert float(v[0, 0].std()) > 1e-6
        assert torch.isfinite(v).all()
    sf.add_state(q, base.nbasis, dims, ens.offsets)
    assert all(np.isfinite(x) and x > 0 for x in sf.result().values())


def test_periodic_shift_equivariance_at_size():
    """A size-independent property on a 256^3 grid (16.8 M cells, 5.9 GB per
    state): on a periodic grid, a forward-Euler stage with a given dt commutes
    with a shift of the cells, bit for bit, in every direction."""
    import torch
    from hermeshd_gb300.solver import Solver
    cfg = config.Config(nx=256, ny=256, nz=256, nbasis=4, iquad=2, ivis=1, coll=2.0, colvis=1.0, ihllc=1)
    s = _solver(cfg)
    q = s.new_state()
    s.init_state(q, 6)                       # fluid at rest, then a smooth periodic perturbation
    k = torch.arange(256, device=q.device, dtype=torch.float64) * (2 * np.pi / 256)
    q[0, 1] += 1e-2 * torch.sin(k)[None, None, :] * torch.cos(2 * k)[None, :, None]
    q[0, 2] += 1e-2 * torch.sin(3 * k)[:, None, None]
    q[1, 0] += 1e-3 * torch.cos(k)[None, None, :]
    dt = 0.5 * s.get_min_dt(q)
    e = s.euler_stage(q.clone(), dt)
    for dim, shift in ((4, 37), (3, -11), (2, 5)):
        es = s.euler_stage(q.roll(shift, dims=dim).contiguous(), dt)
        assert torch.equal(es, e.roll(shift, dims=dim)), dim
    del e, es
    torch.cuda.empty_cache()

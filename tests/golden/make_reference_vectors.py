"""Generate tests/golden/reference/*.npz: outputs of the reference's OWN
routines, executed from its Fortran source by tests/golden/fortran_subset.py
(the reference cannot be compiled here: no Fortran compiler, MPI or MKL).

Routines run as written:
  * initialize.f90  set_basis_function_flags, set_cbasis_3D, init_bf_weights,
                    set_cflm
  * basis_funcs.f90 set_internal_vals_3D, set_face_vals_3D, set_weights_3D
  * flux.f90        flux_calc_pnts_r, flux_hllc, cfcal, limiter, calc_flux_x/y/z,
                    innerintegral2, glflux
  * sources.f90     source_calc
  * prepare_step.f90 exchange_flux;  boundary.f90 apply_boundaries, the
                    periodic, wall, no-slip and outflow routines, and the
                    x-low inflow (x_bc_inflow, set_xlobc_inflow; params.f90 yc)
  * integrator.f90  RK2, RK3, euler_step, prep_advance, calc_rhs,
                    advance_time_level;  hermeshd.f90 get_min_dt
  * src/ces/10_moment/dg_3D_hydro_lqc_SEAN.f90  flux_roe (the Roe variant)
with the module values of params.f90 (variable indices :42-47, sizes :49-62,
floors :93-95, c1d3 ... :73) and of the chosen configuration.  One piece is
restated rather than run: the per-face assembly of calc_flux_x
(flux.f90:226-271: the central flux with cfr = max(cfcal) for ivis 2 and 0
otherwise, then HLLC's rh..en over it), which sits inside the grid loop and
its MPI halo arrays; for the Roe variant rh..en are replaced where kroe > 0.

Fixtures (small, seeded):
  tables_nb{4,8,10}.npz   the basis tables and weights
  limiter_nb{4,8,10}.npz  a state with cells on every limiter branch, before
                          and after the reference's limiter
  faces.npz               face fluxes F(q_L, q_R) of the point flux + HLLC /
                          Roe / central, per direction, ivis 0/1/2, ieos 1/2,
                          for the states of three-cell periodic lines
  ivis2_stage.npz         one ivis-2 forward-Euler stage of the reference into a
                          prefilled output (its rh..en rows stay unwritten)
  step_<case>.npz         the reference's whole step (ReferenceStep): the
                          right-hand side of the initial state and the state,
                          time and time step after the case's steps, in the
                          format of the oracle-written golden fixtures

Run from the repository root:  python tests/golden/make_reference_vectors.py
(add --long [name ...] for the 100-step Sod and vortex fixtures alone)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import fortran_subset as F  # noqa: E402

REF = os.environ.get("HERMESHD_REFERENCE", "/root/reference")
OUT = os.path.join(HERE, "reference")
NBASTOT = 30
IDX = dict(rh=1, mx=2, my=3, mz=4, en=5, pxx=6, pyy=7, pzz=8, pxy=9, pxz=10, pyz=11, nq=11)   # params.f90:42-47
KNAMES = ("kx ky kz kyz kzx kxy kxyz kxx kyy kzz kyzz kzxx kxyy kyyz kzzx kxxy kxxx kyyy kzzz kyyzz kzzxx kxxyy "
          "kyzxx kzxyy kxyzz kxyyzz kyzzxx kzxxyy kxxyyzz").split()


def source(path):
    return open(os.path.join(REF, path)).read()


class Reference:
    """The reference's module state for one (nbasis, iquad) and physics."""

    def __init__(self, nbasis, iquad, ivis=0, ieos=1, aindex=5.0 / 3.0, P_1=0.05, P_base=1.0, rh_floor=5.0e-6,
                 T_floor=1.0, coll=0.0, colvis=0.0):
        nface = iquad * iquad
        npg = nface * iquad
        vals = dict(IDX)
        vals.update(nbastot=NBASTOT, nbasis=nbasis, iquad=iquad, nedge=iquad, nface=nface, npg=npg, nfe=2 * nface,
                    npge=6 * nface, nslim=npg + 6 * nface, aindex=aindex, aindm1=aindex - 1.0, ieos=ieos, ivis=ivis,
                    p_1=P_1, p_base=P_base, rh_floor=rh_floor, t_floor=T_floor, p_floor=T_floor * rh_floor,
                    coll=coll, colvis=colvis, c1d3=1.0 / 3.0, c2d3=2.0 / 3.0, c4d3=4.0 / 3.0, c2d3cv=0.0, c4d3cv=0.0,
                    ibitri=1 if nbasis == 8 else 0, cp=aindex / (aindex - 1.0), pi=np.pi,
                    dxi=1.0, dyi=1.0, dzi=1.0)   # the spacing enters only wgtbf_*, not used here
        vals.update({k: 0 for k in KNAMES})
        A = F.FArray
        vals.update(bfvals_int=A((npg, NBASTOT)), bf_faces=A((npg + 6 * nface, NBASTOT)), xquad=A(20),
                    wgt1d=A(5), wgt2d=A(30), wgt3d=A(100), cbasis=A(NBASTOT),
                    bval_int_wgt=A((npg, NBASTOT)), wgtbf_xmp=A((nface, 2, NBASTOT)),
                    wgtbf_ymp=A((nface, 2, NBASTOT)), wgtbf_zmp=A((nface, 2, NBASTOT)),
                    mxa=A(3), mya=A(3), mza=A(3), kroe=A(nface))
        for side in ("xp", "xm", "yp", "ym", "zp", "zm"):
            vals["bfvals_" + side] = A((nface, NBASTOT))
        vals["mxa"][...] = [2, 3, 4]          # dg_3D_hydro_lqc_SEAN.f90:236-244
        vals["mya"][...] = [3, 4, 2]
        vals["mza"][...] = [4, 2, 3]
        self.ns = ns = F.namespace(vals)
        init, basis, flux = source("src/initialize.f90"), source("src/basis_funcs.f90"), source("src/flux.f90")
        roe = source("src/ces/10_moment/dg_3D_hydro_lqc_SEAN.f90")
        F.translate(init, "set_basis_function_flags", ns)(vals["ibitri"])
        ns["cbasis"][...] = F.translate(init, "set_cbasis_3D", ns)(vals["ibitri"])
        for r in ("set_internal_vals_3D", "set_face_vals_3D", "set_weights_3D"):
            F.translate(basis, r, ns)()
        F.translate(init, "init_bf_weights", ns)(ns["bval_int_wgt"], ns["wgtbf_xmp"], ns["wgtbf_ymp"],
                                                  ns["wgtbf_zmp"])
        self.point_flux = F.translate(flux, "flux_calc_pnts_r", ns)
        self.hllc = F.translate(flux, "flux_hllc", ns)
        self.cfcal = F.translate(flux, "cfcal", ns)
        self.roe = F.translate(roe, "flux_roe", ns)
        self.flux_src = flux
        self.nface, self.nbasis, self.ivis = nface, nbasis, ivis

    def limiter(self, Q):
        """flux.f90:1077-1164 on a Fortran-order Q(nx,ny,nz,nQ,nbasis), in place."""
        nx, ny, nz = Q.shape[:3]
        self.ns.update(nx=nx, ny=ny, nz=nz)
        lim = F.translate(self.flux_src, "limiter", self.ns)
        qa = F.FArray(Q)
        lim(qa)
        return Q

    def face_flux(self, qL, qR, ixyz, solver):
        """The numerical flux of one face whose nface points all carry the
        states qL | qR: the assembly of flux.f90:226-271 over the routines."""
        nf = self.nface
        Qf = F.FArray((2 * nf, 11))
        Qf.a[:nf] = qL
        Qf.a[nf:] = qR
        ff = F.FArray((2 * nf, 11))
        self.point_flux(Qf, ff, ixyz, 2 * nf)
        cfr = np.zeros(nf)
        if self.ivis == 2:
            cw = [self.cfcal(F.FArray(Qf.a[p].copy()), ixyz) for p in range(2 * nf)]
            cfr = np.array([max(cw[p], cw[p + nf]) for p in range(nf)])
        fl = 0.5 * (ff.a[:nf] + ff.a[nf:]) - 0.5 * cfr[:, None] * (Qf.a[nf:] - Qf.a[:nf])
        if solver == "hllc":
            fh = F.FArray((nf, 5))
            self.hllc(Qf, ff, fh, ixyz)
            fl[:, :5] = fh.a
        elif solver == "roe":
            fr = F.FArray((nf, 5))
            self.roe(Qf, ff, fr, ixyz)
            keep = self.ns["kroe"].a > 0
            fl[keep, :5] = fr.a[keep]
        assert np.all(fl == fl[0]), "the face's points carry one state pair"
        return fl[0]


class ReferenceStep(Reference):
    """The reference's whole step on one grid, its routines run as written:
    get_min_dt (hermeshd.f90:145-199), RK2/RK3, euler_step, prep_advance,
    calc_rhs, advance_time_level (integrator.f90), limiter, calc_flux_x/y/z,
    innerintegral2, glflux (flux.f90), source_calc (sources.f90),
    exchange_flux (prepare_step.f90), apply_boundaries and the boundary
    routines (boundary.f90).  Two things stand in for what runs around them:
    the MPI halo exchange of one rank (perform_flux_exchange: a periodic
    direction's neighbour is the rank itself, so the low ghost receives the
    high interior traces and the high ghost the low ones; a bounded
    direction has no neighbour and its ghosts come from the boundary
    routines) and the three lines of step (hermeshd.f90:53-62), which
    update t and dt through scalar arguments."""

    def __init__(self, cfg):
        nb, iq = cfg.nbasis, cfg.iquad
        super().__init__(nb, iq, ivis=cfg.ivis, ieos=cfg.ieos, aindex=cfg.aindex, P_1=cfg.P_1, P_base=cfg.P_base,
                         rh_floor=cfg.rh_floor, T_floor=cfg.T_floor, coll=cfg.coll, colvis=cfg.colvis)
        ns = self.ns
        nx, ny, nz, nf, nq = cfg.nx, cfg.ny, cfg.nz, iq * iq, 11
        A = F.FArray
        ns.update(nx=nx, ny=ny, nz=nz, dxi=nx / cfg.lx, dyi=ny / cfg.ly, dzi=nz / cfg.lz, rh_mult=1.01,
                  ihllc=(cfg.ihllc == 1), llns=False, mpi_p=1, mpi_q=1, mpi_r=1, mpi_nx=1, mpi_ny=1, mpi_nz=1,
                  numprocs=1, iam=0, ierr=0, cartcomm=0, print_mpi=0, mpi_status_size=1, mpi_tt=0,
                  reqs=A(4), stats=A((1, 4)))
        ns["cflm"] = F.translate(source("src/initialize.f90"), "set_cflm", ns)(iq, ns["ibitri"]) \
            if cfg.cflm <= 0 else cfg.cflm
        for name in ("glflux_r", "source_r", "integral_r"):
            ns[name] = A((nx, ny, nz, nq, nb))
        ns.update(flux_x=A((nf, nx + 1, ny, nz, nq)), flux_y=A((nf, nx, ny + 1, nz, nq)),
                  flux_z=A((nf, nx, ny, nz + 1, nq)))
        for d in "xyz":
            ns["cfr" + d] = A((nf, nq))
            ns["qface_" + d] = A((2 * nf, nq))
            ns["fface_" + d] = A((2 * nf, nq))
        for d, sh in (("x", (ny, nz)), ("y", (nx, nz)), ("z", (nx, ny))):
            for end in ("lo", "hi"):
                for part in ("int", "ext"):
                    ns[f"q{d}{end}_{part}"] = A(sh + (nf, nq))

        def noop(*a):
            return None

        for name in ("mpi_barrier", "mpi_isend", "mpi_irecv", "mpi_wait", "mpi_waitall"):
            ns[name] = noop

        def exit_(code):
            raise FloatingPointError("the reference's NaN check ended the run")
        ns["exit"] = exit_
        bc = cfg.bc_names if hasattr(cfg, "bc_names") else (cfg.xlobc, cfg.xhibc, cfg.ylobc, cfg.yhibc, cfg.zlobc,
                                                             cfg.zhibc)
        periodic = [bc[0] == "periodic" and bc[1] == "periodic", bc[2] == "periodic" and bc[3] == "periodic",
                    bc[4] == "periodic" and bc[5] == "periodic"]

        def perform_flux_exchange():
            for k, d in enumerate("xyz"):
                if periodic[k]:
                    ns[f"q{d}lo_ext"].a[...] = ns[f"q{d}hi_int"].a
                    ns[f"q{d}hi_ext"].a[...] = ns[f"q{d}lo_int"].a
        ns["perform_flux_exchange"] = perform_flux_exchange
        bsrc = source("src/boundary.f90")
        for k, (d, end) in enumerate((("x", "lo"), ("x", "hi"), ("y", "lo"), ("y", "hi"), ("z", "lo"), ("z", "hi"))):
            if bc[k] != "inflow":
                ns[f"apply_{d}{end}bc"] = F.translate(bsrc, f"{d}{end}bc_{bc[k]}", ns)
        if bc[0] == "inflow":
            # the parabolic x-low inflow of boundary_custom as apply_boundaries' commented-out call
            # runs it (boundary.f90:759): set_xlobc_inflow once, then x_bc_inflow at every stage
            ns.update(ly=cfg.ly, lyd=-cfg.ly / 2, loc_lyd=-cfg.ly / 2, dy=cfg.ly / ny, mflowrate=0.0,
                      qxlo_ext_def=A((ny, nz, nf, nq)))
            F.translate(source("src/params.f90"), "yc", ns)
            F.translate(bsrc, "set_xlobc_inflow", ns)(cfg.inflow_u, cfg.inflow_rho, cfg.inflow_pressure,
                                                       ns["qxlo_ext_def"])
            inflow = F.translate(bsrc, "x_bc_inflow", ns)
            ns["apply_xlobc"] = lambda qi, qe: inflow(qi, ns["qxlo_ext_def"], qe)
        F.translate(bsrc, "apply_boundaries", ns)
        F.translate(source("src/prepare_step.f90"), "exchange_flux", ns)
        flux = source("src/flux.f90")
        for r in ("limiter", "calc_flux_x", "calc_flux_y", "calc_flux_z", "innerintegral2", "glflux"):
            F.translate(flux, r, ns)
        F.translate(source("src/sources.f90"), "source_calc", ns)
        integ = source("src/integrator.f90")
        for r in ("prep_advance", "calc_rhs", "advance_time_level", "euler_step", "RK2", "RK3"):
            F.translate(integ, r, ns)
        self.get_min_dt = F.translate(source("src/hermeshd.f90"), "get_min_dt", ns)
        self.update = ns["rk2"] if cfg.iorder == 2 else ns["rk3"]
        self.cfg = cfg

    def rhs(self, Q):
        """glflux_r - source_r after prep_advance (the limiter in place)."""
        q = F.FArray(Q)
        self.ns["prep_advance"](q)
        self.ns["calc_rhs"](q)
        return self.ns["glflux_r"].a - self.ns["source_r"].a

    def advance(self, Q, nsteps):
        """nsteps of step (hermeshd.f90:53-62) in place; returns (t, dt)."""
        q = F.FArray(Q)
        q1, q2 = F.FArray(np.zeros_like(Q, order="F")), F.FArray(np.zeros_like(Q, order="F"))
        t = dt = 0.0
        for _ in range(nsteps):
            dt = float(self.get_min_dt(q))
            self.update(q, q1, q2, dt)
            t = t + dt
        return t, dt


class GradFaces(Reference):
    """Face fluxes of the Grad-closure monolith
    (src/ces/10_moment/dg_3D_hydro_bitri_ten_moment.f90), whose ivis 0 is the
    E_ij form (this implementation's ivis 3): its own flux_calc_pnts_r
    (:894-1080), cfcal (:1721-1754) and flux_hllc, assembled as its flux_cal
    does (:1127-1160: the freezing-speed LLF on every variable, HLLC over
    rh..en when ihllc)."""

    def __init__(self, aindex=5.0 / 3.0):
        super().__init__(4, 2, ivis=0, aindex=aindex)
        grad = source("src/ces/10_moment/dg_3D_hydro_bitri_ten_moment.f90")
        self.ns.update(exx=6, eyy=7, ezz=8, exy=9, exz=10, eyz=11, rh_fluid=1.0)
        self.point_flux = F.translate(grad, "flux_calc_pnts_r", self.ns)
        self.cfcal = F.translate(grad, "cfcal", self.ns)
        self.hllc = F.translate(grad, "flux_hllc", self.ns)
        self.ivis = 2          # flux_cal applies the freezing-speed LLF in this form: take that branch below


def faces_grad():
    recs = {"solver": [], "dir": [], "states": [], "fluxes": []}
    g = 5.0 / 3.0
    r = GradFaces(aindex=g)
    rng = np.random.default_rng(300)
    for solver in ("hllc", "central"):
        for d in (1, 2, 3):
            for _ in range(2):
                st = line_states(rng, 2, g)                  # full second moments E_ij
                recs["solver"].append(("central", "hllc").index(solver))
                recs["dir"].append(d)
                recs["states"].append(np.array(st))
                recs["fluxes"].append(np.array([r.face_flux(st[i], st[(i + 1) % 3], d, solver) for i in range(3)]))
    out = {k: np.array(v) for k, v in recs.items()}
    out.update(aindex=g, rh_floor=5.0e-6, T_floor=1.0)
    return out


def grad_source_step():
    """The Grad-closure monolith's implicit source step (source_calc
    :719-790 and advance_time_level_source :839-890), which its RK2 applies
    after each advection stage with one array as input and output
    (:347-348).  Run twice on the same advected state: with distinct input
    and output arrays (every update reads the values before the step), and
    aliased as the monolith calls it (each update reads the ones before it
    in the routine's order).  The advected state is the oracle's RK3 stage
    of the same problem (the monolith's RK3 applies no source step)."""
    sys.path[:0] = [os.path.dirname(os.path.dirname(HERE)), os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                          "oracle")]
    import dataclasses
    import json
    import oracle as O
    from hermeshd_gb300 import config, ic
    cfg = config.Config(nx=4, ny=3, nz=2, nbasis=4, iquad=2, ivis=3, coll=2.0, iorder=2)
    Q = np.asfortranarray(ic.ten_moment_stress(cfg, ic.random_smooth(cfg, seed=9, amp=0.05), p=1.0, amp=0.01))
    o3 = O.Oracle(cfg.replace(iorder=3))
    dt = o3.get_min_dt(Q)
    qgl = o3.euler_step(Q.copy(order="F"), dt)
    r = Reference(4, 2, ivis=0, coll=cfg.coll)
    grad = source("src/ces/10_moment/dg_3D_hydro_bitri_ten_moment.f90")
    r.ns.update(exx=6, eyy=7, ezz=8, exy=9, exz=10, eyz=11, nx=cfg.nx, ny=cfg.ny, nz=cfg.nz, dt=dt,
                source_r=F.FArray((cfg.nx, cfg.ny, cfg.nz, 11, 4)))
    calc = F.translate(grad, "source_calc", r.ns)
    step = F.translate(grad, "advance_time_level_source", r.ns)
    qi = F.FArray(qgl.copy(order="F"))
    calc(qi, 0.0)
    qo = F.FArray(qgl.copy(order="F"))
    step(qi, qo)
    qa = F.FArray(qgl.copy(order="F"))
    calc(qa, 0.0)
    step(qa, qa)
    return dict(Q=Q, dt=dt, Q_advected=qgl, separate=qo.a, aliased=qa.a,
                config=json.dumps(dataclasses.asdict(cfg), sort_keys=True))


def initial_state(cfg, icid, vis=0.1):
    """set_ic (initialcon.f90:20-72) for problems 1-5 (isentropic vortex v0,
    v1; Sod v0, v1; Poiseuille's fluid at rest), with params.f90's cell
    centres xc, yc, zc on the centred domain (initialize.f90:310-326)."""
    r = Reference(cfg.nbasis, cfg.iquad, ivis=cfg.ivis, aindex=cfg.aindex, P_base=cfg.P_base,
                  rh_floor=cfg.rh_floor, T_floor=cfg.T_floor, coll=cfg.coll, colvis=cfg.colvis)
    ns = r.ns
    ns.update(nx=cfg.nx, ny=cfg.ny, nz=cfg.nz, lx=cfg.lx, ly=cfg.ly, lz=cfg.lz,
              lxd=-cfg.lx / 2, lyd=-cfg.ly / 2, lzd=-cfg.lz / 2, loc_lxd=-cfg.lx / 2, loc_lyd=-cfg.ly / 2,
              loc_lzd=-cfg.lz / 2, dx=cfg.lx / cfg.nx, dy=cfg.ly / cfg.ny, dz=cfg.lz / cfg.nz, vis=vis,
              mflowrate=0.0, iam=0, qxlo_ext_def=F.FArray((cfg.ny, cfg.nz, cfg.iquad ** 2, 11)),
              mpi_print=lambda *a: None)
    params = source("src/params.f90")
    for f in ("xc", "yc", "zc"):
        F.translate(params, f, ns)
    F.translate(source("src/boundary.f90"), "set_xlobc_inflow", ns)
    ic_src = source("src/initialcon.f90")
    for f in ("isentropic_vortex", "sod_shock_tube_1d", "poiseuille_flow", "set_ic"):
        F.translate(ic_src, f, ns)
    Q = F.FArray((cfg.nx, cfg.ny, cfg.nz, 11, cfg.nbasis))
    ns["set_ic"](Q, icid)
    return Q.a


def initial_states():
    sys.path[:0] = [os.path.dirname(os.path.dirname(HERE))]
    import dataclasses
    import json
    from hermeshd_gb300 import config
    out = {}
    for icid in (1, 2, 3, 4, 5):
        if icid in (1, 2):
            cfg = config.isentropic_vortex_2d(n=12)
        elif icid in (3, 4):
            cfg = config.Config(nx=16, ny=6, nz=1, nbasis=4, iquad=2, lx=1.0, ly=0.5, P_base=1.0)
        else:
            cfg = config.Config(nx=6, ny=8, nz=1, nbasis=4, iquad=2, ivis=1, coll=10.0, colvis=1.0)
        out[f"Q_{icid}"] = initial_state(cfg, icid)
        out[f"config_{icid}"] = json.dumps(dataclasses.asdict(cfg), sort_keys=True)
    return out


def tables(nb, iq):
    r = Reference(nb, iq)
    ns = r.ns
    npg, nf = iq ** 3, iq * iq
    out = {k: ns[k].a[:, :nb].copy() for k in ("bfvals_int", "bf_faces", "bfvals_xp", "bfvals_xm", "bfvals_yp",
                                               "bfvals_ym", "bfvals_zp", "bfvals_zm", "bval_int_wgt")}
    out["wgt3d"] = ns["wgt3d"].a[:npg].copy()
    out["wgt2d"] = ns["wgt2d"].a[:nf].copy()
    out["cbasis"] = ns["cbasis"].a[:nb].copy()
    return out


def floored_state(nb, iq, seed, shape=(4, 3, 2), rh_floor=0.4, T_floor=0.5):
    """Cells on every branch of the limiter: an average below the density
    floor, face densities below it, an average pressure below the pressure
    floor, face pressures below it, and cells left alone."""
    rng = np.random.default_rng(seed)
    Q = np.zeros(shape + (11, nb), order="F")
    Q[..., 0, 0] = 1.0 + 0.05 * rng.standard_normal(shape)
    Q[..., 1:4, 0] = 0.05 * rng.standard_normal(shape + (3,))
    Q[..., 4, 0] = 1.5 + 0.05 * rng.standard_normal(shape)
    Q[..., :5, 1:] = 0.2 * rng.standard_normal(shape + (5, nb - 1))
    Q[0, 0, 0, 0, 0] = 0.35                                  # average density below the floor
    m2 = (Q[1, 0, 0, 1:4, 0] ** 2).sum()
    Q[1, 0, 0, 4, 0] = 0.5 * m2 / Q[1, 0, 0, 0, 0] + 0.1    # average pressure below the floor
    Q[2, 0, 0, 0, 1:] = 0.5                                  # face densities below the floor
    Q[3, 1, 0, 4, 1:] = 0.6                                  # face pressures below the floor
    return Q, rh_floor, T_floor


def line_states(rng, ivis, g, n=3):
    out = []
    for _ in range(n):
        rho, v, p = rng.uniform(0.5, 2.0), rng.uniform(-1.0, 1.0, 3), rng.uniform(0.5, 2.0)
        q = np.zeros(11)
        q[0], q[1:4] = rho, rho * v
        q[4] = p / (g - 1) + 0.5 * rho * v @ v
        dev = rng.uniform(-0.1, 0.1, 6)
        if ivis == 2:
            for k, (a, b) in enumerate(((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))):
                q[5 + k] = rho * v[a] * v[b] + (p if a == b else 0.0) + dev[k]
        else:
            q[5:] = dev
        out.append(q)
    return out


FACE_CASES = [   # ivis, ieos, solver
    (0, 1, "hllc"), (1, 1, "hllc"), (2, 1, "hllc"), (0, 1, "central"), (2, 1, "central"),
    (0, 2, "hllc"), (1, 2, "central"), (0, 1, "roe"), (1, 1, "roe"),
]


def faces():
    recs = {"ivis": [], "ieos": [], "solver": [], "dir": [], "states": [], "fluxes": []}
    g, P_1, P_base, colvis = 5.0 / 3.0, 0.05, 1.0, 0.3
    for c, (ivis, ieos, solver) in enumerate(FACE_CASES):
        r = Reference(4, 2, ivis=ivis, ieos=ieos, aindex=g, P_1=P_1, P_base=P_base, colvis=colvis)
        rng = np.random.default_rng(100 + c)
        for d in (1, 2, 3):
            for _ in range(2):
                st = line_states(rng, ivis, g)
                fl = [r.face_flux(st[i], st[(i + 1) % 3], d, solver) for i in range(3)]
                recs["ivis"].append(ivis)
                recs["ieos"].append(ieos)
                recs["solver"].append(("central", "hllc", "roe").index(solver))
                recs["dir"].append(d)
                recs["states"].append(np.array(st))
                recs["fluxes"].append(np.array(fl))
    out = {k: np.array(v) for k, v in recs.items()}
    out.update(aindex=g, P_1=P_1, P_base=P_base, colvis=colvis, rh_floor=5.0e-6, T_floor=1.0)
    return out


def step_cases():
    """name -> (Config, initial state, steps): the configurations of the
    oracle-written golden fixtures that the reference's modular code covers
    (not its ivis-2 update, which leaves rh..en unwritten, nor the Roe and
    Grad-closure variants, the stochastic stress or the body force)."""
    sys.path[:0] = [os.path.dirname(os.path.dirname(HERE))]
    from hermeshd_gb300 import config, ic
    c = {}
    cfg = config.sod_1d(nx=32)
    c["sod_32_hllc_rk2_nb4"] = (cfg, ic.sod(cfg), 20)
    cfg = config.isentropic_vortex_2d(n=8)
    c["vortex_8_rk3_nb10"] = (cfg, ic.isentropic_vortex(cfg), 10)
    cfg = config.taylor_green_3d(n=4, precision="fp64")
    c["tgv_4_ivis1_rk3_nb4"] = (cfg, ic.taylor_green(cfg, perturb=1e-3, seed=1), 10)
    cfg = config.Config(nx=4, ny=3, nz=2, nbasis=8, iquad=2, ivis=1, coll=2.0, colvis=0.5,
                        xlobc="wall", xhibc="noslip", zlobc="outflow", zhibc="wall")
    c["walls_nb8_ivis1_rk2"] = (cfg, ic.random_smooth(cfg, seed=5, amp=0.05, stress_amp=0.01), 10)
    # no oracle-written twins: the ivis-0 relaxation source, and the Tait EOS with HLLC at walls
    cfg = config.Config(nx=4, ny=3, nz=2, nbasis=4, iquad=2, ivis=0, coll=0.8, colvis=0.0, iorder=3)
    c["relax_ivis0_rk3_nb4"] = (cfg, ic.random_smooth(cfg, seed=7, amp=0.08, stress_amp=0.05), 8)
    cfg = config.Config(nx=6, ny=4, nz=1, nbasis=4, iquad=2, ieos=2, P_1=0.05, P_base=1.0, xlobc="wall",
                        xhibc="noslip")
    c["tait_walls_rk2_nb4"] = (cfg, ic.random_smooth(cfg, seed=4, amp=0.05), 10)
    cfg = config.Config(nx=6, ny=4, nz=1, lx=1.5, ly=1.0, nbasis=4, iquad=2, ivis=1, coll=3.0, colvis=1.0,
                        xlobc="inflow", xhibc="wall", ylobc="noslip", yhibc="noslip", inflow_u=0.3, inflow_p=1.0)
    c["inflow_channel_rk2_nb4"] = (cfg, ic.channel(cfg, amplitude=1e-3, seed=0), 6)
    cfg = config.Config(nx=4, ny=3, nz=2, nbasis=10, iquad=3, ivis=1, coll=2.0, colvis=0.5, ieos=2, P_1=0.05,
                        P_base=1.0, iorder=3, xlobc="wall", xhibc="noslip", ylobc="outflow", yhibc="outflow")
    c["mixed_nb10_ivis1_tait_rk3"] = (cfg, ic.random_smooth(cfg, seed=8, amp=0.04, stress_amp=0.01), 4)
    return c


def step_fixture(cfg, Q0, steps):
    import dataclasses
    import json
    Q0 = np.asfortranarray(Q0)
    r = ReferenceStep(cfg)
    rhs = r.rhs(Q0.copy(order="F"))
    Q = Q0.copy(order="F")
    t, dt = r.advance(Q, steps)
    return dict(Q0=Q0, rhs=rhs, Q=Q, t=t, dt=dt, steps=steps,
                config=json.dumps(dataclasses.asdict(cfg), sort_keys=True))


def ivis2_stage():
    """One euler_step of the reference with ivis 2, into a Q_out prefilled
    with 7.0: integrator.f90:181-228 writes only the stress rows."""
    sys.path[:0] = [os.path.dirname(os.path.dirname(HERE))]
    import dataclasses
    import json
    from hermeshd_gb300 import config, ic
    cfg = config.Config(nx=4, ny=3, nz=2, nbasis=4, iquad=2, ivis=2, coll=1.5, colvis=1.0)
    Q = np.asfortranarray(ic.ten_moment_stress(cfg, ic.random_smooth(cfg, seed=3, amp=0.05), p=1.0, amp=0.01))
    r = ReferenceStep(cfg)
    dt = float(r.get_min_dt(F.FArray(Q.copy(order="F"))))
    qin = F.FArray(Q.copy(order="F"))
    qout = F.FArray(np.full_like(Q, 7.0, order="F"))
    r.ns["euler_step"](qin, qout, dt)
    return dict(Q_in=Q, dt=dt, Q_out=qout.a, config=json.dumps(dataclasses.asdict(cfg), sort_keys=True))


def long_cases():
    """The Sod tube of the 100-step parity bar (256 cells, nb 4, HLLC, RK2):
    about 15 minutes of the executed reference (`--long`)."""
    sys.path[:0] = [os.path.dirname(os.path.dirname(HERE))]
    from hermeshd_gb300 import config, ic
    cfg = config.sod_1d(nx=256)
    c = {"sod_256_hllc_rk2_nb4_100": (cfg, ic.sod(cfg), 100)}
    cfg = config.isentropic_vortex_2d(n=16)
    c["vortex_16_rk3_nb10_100"] = (cfg, ic.isentropic_vortex(cfg), 100)   # about an hour
    return c


def main():
    os.makedirs(OUT, exist_ok=True)
    if "--long" in sys.argv:
        only = [a for a in sys.argv[1:] if not a.startswith("--")]
        for name, (cfg, Q0, steps) in long_cases().items():
            if only and not any(o in name for o in only):
                continue
            np.savez_compressed(os.path.join(OUT, f"step_{name}.npz"), **step_fixture(cfg, Q0, steps))
        return
    np.savez_compressed(os.path.join(OUT, "ivis2_stage.npz"), **ivis2_stage())
    for name, (cfg, Q0, steps) in step_cases().items():
        np.savez_compressed(os.path.join(OUT, f"step_{name}.npz"), **step_fixture(cfg, Q0, steps))
    for nb, iq in ((4, 2), (8, 2), (10, 3)):
        np.savez_compressed(os.path.join(OUT, f"tables_nb{nb}.npz"), **tables(nb, iq))
        Q, rf, tf = floored_state(nb, iq, seed=nb)
        r = Reference(nb, iq, rh_floor=rf, T_floor=tf)
        after = r.limiter(Q.copy(order="F"))
        np.savez_compressed(os.path.join(OUT, f"limiter_nb{nb}.npz"), before=Q, after=after, rh_floor=rf, T_floor=tf,
                 aindex=5.0 / 3.0)
    np.savez_compressed(os.path.join(OUT, "faces.npz"), **faces())
    np.savez_compressed(os.path.join(OUT, "faces_grad.npz"), **faces_grad())
    np.savez_compressed(os.path.join(OUT, "grad_source_step.npz"), **grad_source_step())
    np.savez_compressed(os.path.join(OUT, "initial_states.npz"), **initial_states())


if __name__ == "__main__":
    main()

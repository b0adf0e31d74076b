"""The whole right-hand side restated a second time in numpy, against the C
oracle, on 3-D grids with every basis mode populated: periodic, and with the
wall, no-slip, outflow and x-lo inflow boundaries (boundary.f90:76-338 on the traces that
prepare_step.f90:20-41 hands them).

Independent of the oracle's tables and loops: the basis is evaluated here
from its definition (initialize.f90:126-217: the families {1, x, y, z},
{1, x, y, z, yz, zx, xy, xyz} and {1, x, y, z, yz, zx, xy, P2(x), P2(y),
P2(z)} of unnormalised Legendre products with cbasis = prod(2k + 1)), and the
operator is written in its general form

  glflux_b = 1/4 cbasis_b sum_d dxi_d [ sum_faces w2 (phi_b(+) F_d,hi - phi_b(-) F_d,lo)
                                        - sum_points w3 d phi_b/ds_d f_d(Q) ]
  source_b = 1/8 cbasis_b sum_points w3 phi_b S(Q)

which flux.f90:751-928 (innerintegral2, written out row by row for each basis
function) and flux.f90:958-972 (glflux) and sources.f90:70-76 spell out.  The
face fluxes come from the per-state restatement of flux.f90 in
test_oracle_face_restatement.py.  The C oracle evaluates the same operator
through its own tables (basis_funcs.f90's bfvals_*), loops and reductions,
so agreement to rounding (measured 1e-15 to 6e-15 of each variable's scale)
checks the volume and surface integrals, the face traces, the ghost traces
and the sources for nb 4/8/10, ivis 0/1/2/3 (3: the Grad closure of the
monolithic 10-moment code), the central, HLLC and Roe fluxes,
and the Tait EOS with HLLC's stale 1/rho taken from the right state at each
face's last point."""
import numpy as np
import pytest

from hermeshd_gb300 import config, ic

from test_oracle_face_restatement import MX, MZ, face_flux, point_flux, source, stress_sample

NQ = 11
FAMILIES = {
    4: [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)],
    8: [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (0, 1, 1), (1, 0, 1), (1, 1, 0), (1, 1, 1)],
    10: [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (0, 1, 1), (1, 0, 1), (1, 1, 0), (2, 0, 0), (0, 2, 0),
         (0, 0, 2)],
}


def leg(k, s):
    return (1.0, s, 1.5 * s * s - 0.5)[k]


def dleg(k, s):
    return (0.0, 1.0, 3.0 * s)[k]


def phi(fam, p):
    return leg(fam[0], p[0]) * leg(fam[1], p[1]) * leg(fam[2], p[2])


def dphi(fam, p, d):
    out = 1.0
    for a in range(3):
        out *= dleg(fam[a], p[a]) if a == d else leg(fam[a], p[a])
    return out


def rule(iquad):
    s, w = np.polynomial.legendre.leggauss(iquad)
    return list(s), list(w)


def ghost(kind, side, d, interior, cfg=None, cell=None):
    """Ghost traces of one boundary face from the interior traces at its
    points (boundary.f90:76-338): no-slip zeroes every momentum, a wall the
    normal one; outflow copies the trace and zeroes the normal momentum of
    all the face's points when any of them flows in (lo: a positive maximum;
    y/z hi: a negative minimum).  The x-hi outflow routine never copies the
    trace, so its ghost keeps the zeros it started from.  The x-lo inflow
    (x_bc_inflow with set_xlobc_inflow's profile, boundary.f90:568-612)
    copies the trace and sets rho, m_x, E from the parabolic stream at the
    cell centre's height, m_y = m_z = 0."""
    m = MX + d
    out = [q.copy() for q in interior]
    if kind == "inflow":
        assert side == "lo" and d == 0
        yp = (cell[1] + 0.5) * cfg.ly / cfg.ny                 # yc(j) - lyd
        vx = 4 * cfg.inflow_u * yp * (cfg.ly - yp) / cfg.ly ** 2
        den = cfg.inflow_rho
        pres = cfg.inflow_p if cfg.inflow_p > 0 else den * cfg.T_floor
        for q in out:
            q[0], q[MX], q[MX + 1], q[MX + 2] = den, den * vx, 0.0, 0.0
            q[MZ + 1] = pres / (cfg.aindex - 1) + 0.5 * den * vx ** 2
    elif kind == "noslip":
        for q in out:
            q[MX:MZ + 1] = 0.0
    elif kind == "wall":
        for q in out:
            q[m] = 0.0
    elif kind == "outflow":
        if side == "hi" and d == 0:
            return [np.zeros(NQ) for _ in interior]
        normal = [q[m] for q in out]
        if (side == "lo" and max(normal) > 0.0) or (side == "hi" and min(normal) < 0.0):
            for q in out:
                q[m] = 0.0
    else:
        raise ValueError(kind)
    return out


def restated_rhs(cfg, Q, step=0, stage=0):
    """glflux - source (the oracle's rhs without the limiter), shape of Q;
    with the stochastic stress (cfg.llns) the draws of the given step and
    stage.  Noise sites: cell i + nx (j + ny k) for the interior calls (one
    independent draw per direction's call, kinds 3-5); for the faces of
    direction d (kinds 0-2) the face's index on the grid of faces, where a
    direction periodic at both ends has n planes (the face at n is the face
    at 0); points: the interior point index, and for faces the left states'
    points 0..nface-1 and the right states' nface..2 nface-1, in the
    reference's face-point order (basis_funcs.f90:392-423)."""
    bcs = ((cfg.xlobc, cfg.xhibc), (cfg.ylobc, cfg.yhibc), (cfg.zlobc, cfg.zhibc))
    fams = FAMILIES[cfg.nbasis]
    nb = len(fams)
    cb = [float((2 * a + 1) * (2 * b + 1) * (2 * c + 1)) for a, b, c in fams]
    s, w = rule(cfg.iquad)
    n = (cfg.nx, cfg.ny, cfg.nz)
    dxi = (cfg.nx / cfg.lx, cfg.ny / cfg.ly, cfg.nz / cfg.lz)
    interior = [((s[a], s[b], s[c]), w[a] * w[b] * w[c]) for a in range(len(s)) for b in range(len(s))
                for c in range(len(s))]

    cache = {}
    cbv = np.array(cb)

    def basis(p):
        key = tuple(p)
        if key not in cache:
            cache[key] = np.array([phi(f, p) for f in fams])
        return cache[key]

    def value(cell, p):
        return Q[cell] @ basis(p)

    # d phi_b / ds_d at the interior points, times dxi_d: (npg, 3, nb)
    dphi_int = np.array([[[dxi[d] * dphi(f, p, d) for f in fams] for d in range(3)] for p, _ in interior])

    nf = len(s) ** 2
    periodic = [bcs[d][0] == "periodic" and bcs[d][1] == "periodic" for d in range(3)]

    def noise(kind, site, pt):
        return stress_sample(cfg, step, stage, kind, site, pt) if cfg.llns else None

    def face_site(d, face):
        """face = (i, j, k) with the index along d running 0..n[d]"""
        f = list(face)
        ext = [n[0], n[1], n[2]]
        if periodic[d]:
            f[d] %= n[d]
        else:
            ext[d] += 1
        return f[0] + ext[0] * (f[1] + ext[1] * f[2])

    out = np.zeros_like(Q)
    for i in range(n[0]):
        for j in range(n[1]):
            for k in range(n[2]):
                cell = (i, j, k)
                g = np.zeros((NQ, nb))
                src = np.zeros((NQ, nb))
                site = i + n[0] * (j + n[1] * k)
                # volume terms and sources at the interior points
                for gi, (p, wp) in enumerate(interior):
                    q = value(cell, p)
                    f = np.array([point_flux(cfg, q, d, noise(3 + d, site, gi)) for d in range(3)])  # (3, NQ)
                    g -= 0.25 * wp * (f.T @ dphi_int[gi]) * cbv
                    src += 0.125 * wp * np.outer(source(cfg, q), basis(p)) * cbv
                # surface terms: the hi and lo faces of each direction
                for d in range(3):
                    t1, t2 = [a for a in range(3) if a != d]
                    up = list(cell)
                    up[d] = (up[d] + 1) % n[d]
                    dn = list(cell)
                    dn[d] = (dn[d] - 1) % n[d]
                    # face points in the reference's order: point o * ne + m has the
                    # coordinates (y, z) = (m, o) on x faces, (x, z) = (o, m) on y
                    # faces, (x, y) = (m, o) on z faces
                    pts = []
                    for o in range(len(s)):
                        for m in range(len(s)):
                            hi = [0.0] * 3
                            lo = [0.0] * 3
                            hi[d], lo[d] = 1.0, -1.0
                            a, c = (m, o) if d != 1 else (o, m)
                            hi[t1] = lo[t1] = s[a]
                            hi[t2] = lo[t2] = s[c]
                            pts.append((hi, lo, w[a] * w[c]))
                    f_hi = list(cell)
                    f_hi[d] += 1
                    s_hi, s_lo = face_site(d, f_hi), face_site(d, cell)
                    # neighbour traces, or the boundary's ghost traces at the domain's ends
                    if cell[d] == n[d] - 1 and bcs[d][1] != "periodic":
                        right = ghost(bcs[d][1], "hi", d, [value(cell, hi) for hi, _, _ in pts])
                    else:
                        right = [value(tuple(up), lo) for _, lo, _ in pts]
                    if cell[d] == 0 and bcs[d][0] != "periodic":
                        left = ghost(bcs[d][0], "lo", d, [value(cell, lo) for _, lo, _ in pts], cfg, cell)
                    else:
                        left = [value(tuple(dn), hi) for hi, _, _ in pts]
                    # the Tait sound speeds' stale 1/rho: the right state at the face's last
                    # point, (s_max, s_max) in the reference's point order (basis_funcs.f90:392-423)
                    r_hi, r_lo = right[-1][0], value(cell, pts[-1][1])[0]
                    for m, (hi, lo, w2) in enumerate(pts):
                        F_hi, _ = face_flux(cfg, value(cell, hi), right[m], d, rho_last=r_hi,
                                            SL=noise(d, s_hi, m), SR=noise(d, s_hi, nf + m))
                        F_lo, _ = face_flux(cfg, left[m], value(cell, lo), d, rho_last=r_lo,
                                            SL=noise(d, s_lo, m), SR=noise(d, s_lo, nf + m))
                        g += 0.25 * dxi[d] * w2 * (np.outer(F_hi, basis(hi)) - np.outer(F_lo, basis(lo))) * cbv
                out[i, j, k] = g - src
    return out


CASES = [
    # nb, iquad, ivis, ihllc, ieos
    (4, 2, 0, 1, 1),
    (4, 2, 1, 2, 1),
    (8, 2, 1, 1, 1),
    (8, 2, 2, 0, 1),
    (10, 3, 0, 2, 1),
    (10, 3, 2, 1, 1),
    (10, 3, 1, 0, 1),
    (4, 2, 0, 1, 2),
    (10, 3, 1, 1, 2),
    (8, 2, 2, 0, 2),
    (4, 2, 3, 1, 1),
    (10, 3, 3, 0, 1),
    (8, 2, 3, 2, 1),
]


@pytest.mark.parametrize("nb,iq,ivis,ihllc,ieos", CASES,
                         ids=["nb%d_ivis%d_%s%s" % (c[0], c[2], ("central", "hllc", "roe")[c[3]],
                                                    "_tait" if c[4] == 2 else "") for c in CASES])
def test_rhs_matches_the_general_form(nb, iq, ivis, ihllc, ieos):
    import oracle as O
    cfg = config.Config(nx=3, ny=2, nz=2, nbasis=nb, iquad=iq, ivis=ivis, ieos=ieos, ihllc=ihllc,
                        coll=0.0 if ivis == 1 else 0.8, colvis=0.3, lx=1.5, ly=0.8, lz=1.1, P_1=0.05, P_base=1.0)
    Q = ic.random_smooth(cfg, seed=10 * nb + ivis, amp=0.2, stress_amp=0.05)
    if ivis >= 2:
        ic.ten_moment_stress(cfg, Q, p=1.0, amp=0.05, seed=nb)
    Q = np.asfortranarray(Q)
    got = O.Oracle(cfg).rhs(Q.copy(order="F"), limit=False)
    want = restated_rhs(cfg, Q)
    scale = np.abs(want).max(axis=(0, 1, 2, 4), keepdims=True)      # per variable
    err = np.abs(got - want) / np.maximum(scale, 1e-300)
    assert err.max() <= 1e-12, (err.max(), np.unravel_index(err.argmax(), err.shape))
    assert np.abs(want[..., 1:]).max() > 1e-3 * np.abs(want).max()   # the higher modes carry weight


BC_CASES = [
    # nb, iquad, ivis, ihllc, boundaries (x lo/hi, y lo/hi, z lo/hi)
    (8, 2, 1, 1, ("periodic", "periodic", "wall", "wall", "periodic", "periodic")),
    (4, 2, 1, 2, ("periodic", "periodic", "noslip", "noslip", "periodic", "periodic")),
    (4, 2, 0, 1, ("outflow", "periodic", "outflow", "outflow", "outflow", "outflow")),
    (10, 3, 2, 1, ("wall", "wall", "outflow", "noslip", "noslip", "wall")),
    (8, 2, 1, 2, ("inflow", "wall", "noslip", "noslip", "periodic", "periodic")),
]


@pytest.mark.parametrize("nb,iq,ivis,ihllc,bc", BC_CASES, ids=["walls_y_nb8", "noslip_y_nb4_roe", "outflow_nb4",
                                                                "mixed_nb10_ivis2", "inflow_channel_nb8"])
def test_rhs_with_boundaries(nb, iq, ivis, ihllc, bc):
    """The ghost traces of the wall, no-slip and outflow boundaries (outflow
    states on both sides of the normal-velocity sign, so both of its branches
    run), in the general form."""
    import oracle as O
    cfg = config.Config(nx=3, ny=3, nz=2, nbasis=nb, iquad=iq, ivis=ivis, ieos=1, ihllc=ihllc,
                        coll=0.0 if ivis == 1 else 0.8, colvis=0.3, lx=1.5, ly=1.2, lz=1.1,
                        xlobc=bc[0], xhibc=bc[1], ylobc=bc[2], yhibc=bc[3], zlobc=bc[4], zhibc=bc[5],
                        inflow_u=0.4, inflow_rho=1.1, inflow_p=0.9)
    Q = ic.random_smooth(cfg, seed=7 * nb + ivis, amp=0.2, stress_amp=0.05)
    if ivis == 2:
        ic.ten_moment_stress(cfg, Q, p=1.0, amp=0.05, seed=nb)
    Q = np.asfortranarray(Q)
    got = O.Oracle(cfg).rhs(Q.copy(order="F"), limit=False)
    want = restated_rhs(cfg, Q)
    scale = np.abs(want).max(axis=(0, 1, 2, 4), keepdims=True)
    err = np.abs(got - want) / np.maximum(scale, 1e-300)
    assert err.max() <= 1e-12, (err.max(), np.unravel_index(err.argmax(), err.shape))


NOISE_CASES = [
    # nb, iquad, ivis, ihllc, boundaries x, y, z (lo = hi), step, stage
    (4, 2, 1, 2, ("periodic", "periodic", "periodic"), 0, 0),
    (8, 2, 0, 1, ("wall", "periodic", "noslip"), 5, 1),
    (10, 3, 2, 0, ("periodic", "wall", "periodic"), 2 ** 33 + 3, 2),
]


@pytest.mark.parametrize("nb,iq,ivis,ihllc,bc,step,stage", NOISE_CASES, ids=["nb4_roe_periodic", "nb8_hllc_walls",
                                                                            "nb10_ivis2_central"])
def test_rhs_with_the_stochastic_stress(nb, iq, ivis, ihllc, bc, step, stage):
    """The stochastic stress restated from its counter scheme and placed in the
    point flux as flux.f90:85-100 does (momentum - S, energy - S.v; no S in the
    10-moment momentum and stress fluxes), at every face side and interior
    call, against the oracle at a given step and stage."""
    import oracle as O
    cfg = config.Config(nx=3, ny=2, nz=2, nbasis=nb, iquad=iq, ivis=ivis, ieos=1, ihllc=ihllc,
                        coll=0.0 if ivis == 1 else 0.8, colvis=0.3, lx=1.5, ly=0.8, lz=1.1,
                        xlobc=bc[0], xhibc=bc[0], ylobc=bc[1], yhibc=bc[1], zlobc=bc[2], zhibc=bc[2],
                        llns=True, eta_sd=0.05, zeta_sd=0.02, seed=(3 << 32) + 11)
    Q = ic.random_smooth(cfg, seed=nb, amp=0.2, stress_amp=0.05)
    if ivis >= 2:
        ic.ten_moment_stress(cfg, Q, p=1.0, amp=0.05, seed=nb)
    Q = np.asfortranarray(Q)
    o = O.Oracle(cfg)
    o.set_noise_counter(step)
    for _ in range(stage):                 # the stage counter advances with each forward-Euler stage
        o.euler_step(Q.copy(order="F"), 1e-6)
    got = o.rhs(Q.copy(order="F"), limit=False)
    want = restated_rhs(cfg, Q, step, stage)
    quiet = restated_rhs(cfg.replace(llns=False), Q)
    scale = np.abs(want).max(axis=(0, 1, 2, 4), keepdims=True)
    err = np.abs(got - want) / np.maximum(scale, 1e-300)
    assert err.max() <= 1e-12, (err.max(), np.unravel_index(err.argmax(), err.shape))
    assert np.abs(want - quiet).max() > 1e-3 * np.abs(want).max()   # the stress moved the result

"""Generate dg_tables_gen.cuh: the Legendre basis / Gauss quadrature tables
of each supported (nbasis, iquad) pair as compile-time constants.

The values are computed with the same double-precision operations, in the
same order, as the reference's table setup (basis_funcs.f90:265-627,
initialize.f90:126-220,350-389), so the face, interior and limiter tables are
bit-identical to the ones the oracle builds at run time
(tests/test_oracle_kat.py::test_generated_tables_bit_identical checks
this).  Combined tables (volume, surface and source quadrature weights) fold
the constant factors 0.25*cbasis*w, and are used by the kernels with every
zero entry skipped at compile time.

Run:  python gen_tables.py  (writes dg_tables_gen.cuh next to this file)
"""
from __future__ import annotations

import math
import os

# basis families as (degree in x, degree in y, degree in z), in the index
# order of initialize.f90:126-194 for the supported pairs
FAMILIES = {
    # ibitri 0, iquad 2: {1, x, y, z}
    (4, 2): [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)],
    # ibitri 1, iquad 2: {1, x, y, z, yz, zx, xy, xyz}
    (8, 2): [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (0, 1, 1), (1, 0, 1), (1, 1, 0), (1, 1, 1)],
    # ibitri 0, iquad 3: {1, x, y, z, yz, zx, xy, P2(x), P2(y), P2(z)}
    (10, 3): [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (0, 1, 1), (1, 0, 1), (1, 1, 0),
              (2, 0, 0), (0, 2, 0), (0, 0, 2)],
}


def xquad(iquad):
    """basis_funcs.f90:284-302."""
    if iquad == 2:
        c = 1.0 / math.sqrt(3.0)
        return [-c, c]
    if iquad == 3:
        c = math.sqrt(15.0) / 5.0
        return [-c, 0.0, c]
    raise ValueError(iquad)


def wgt1d(iquad):
    """basis_funcs.f90:578-596."""
    if iquad == 2:
        return [1.0, 1.0]
    if iquad == 3:
        return [5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0]
    raise ValueError(iquad)


def wgt2d(iquad):
    ne, w1 = iquad, wgt1d(iquad)
    if iquad == 2:
        return [1.0] * 4
    return [w1[m] * w1[i] for i in range(ne) for m in range(ne)]


def wgt3d(iquad):
    ne, w1, w2 = iquad, wgt1d(iquad), wgt2d(iquad)
    if iquad == 2:
        return [1.0] * 8
    return [w2[r] * w1[i] for i in range(ne) for r in range(ne * ne)]


def L(deg, s):
    if deg == 0:
        return 1.0
    if deg == 1:
        return s
    return 1.5 * (s * s) - 0.5     # basis_funcs.f90:307


def dL(deg, s):
    if deg == 0:
        return 0.0
    if deg == 1:
        return 1.0
    return 3.0 * s                 # flux.f90:820-822 (3*bfvals_int(kx))


def phi(fam, x, y, z):
    ex, ey, ez = fam
    return (L(ex, x) * L(ey, y)) * L(ez, z)


def cbasis(fam):
    ex, ey, ez = fam
    return float((2 * ex + 1) * (2 * ey + 1) * (2 * ez + 1))   # initialize.f90:206-217


def points(iquad):
    xq, ne = xquad(iquad), iquad
    interior = [(xq[ix], xq[iy], xq[iz]) for ix in range(ne) for iy in range(ne) for iz in range(ne)]
    # face point p = i*ne + m: zp has x = xq[m], y = xq[i]; yp has x = xq[i],
    # z = xq[m]; xp has y = xq[m], z = xq[i] (basis_funcs.f90:392-423)
    face = {}
    face["xp"] = [(1.0, xq[m], xq[i]) for i in range(ne) for m in range(ne)]
    face["xm"] = [(-1.0, xq[m], xq[i]) for i in range(ne) for m in range(ne)]
    face["yp"] = [(xq[i], 1.0, xq[m]) for i in range(ne) for m in range(ne)]
    face["ym"] = [(xq[i], -1.0, xq[m]) for i in range(ne) for m in range(ne)]
    face["zp"] = [(xq[m], xq[i], 1.0) for i in range(ne) for m in range(ne)]
    face["zm"] = [(xq[m], xq[i], -1.0) for i in range(ne) for m in range(ne)]
    return interior, face


def tables(nb, iquad):
    fams = FAMILIES[(nb, iquad)]
    interior, face = points(iquad)
    w2, w3 = wgt2d(iquad), wgt3d(iquad)
    T = {}
    T["INT"] = [[phi(f, *pt) for f in fams] for pt in interior]
    for k in ("xp", "xm", "yp", "ym", "zp", "zm"):
        T[k.upper()] = [[phi(f, *pt) for f in fams] for pt in face[k]]
    # bf_faces rows 1..npge: xm, xp, ym, yp, zm, zp (basis_funcs.f90:527-536)
    T["LIM"] = T["XM"] + T["XP"] + T["YM"] + T["YP"] + T["ZM"] + T["ZP"]
    cb = [cbasis(f) for f in fams]
    # volume quadrature: 0.25*cbasis(b)*w3d(g)*dphi_b/dxi_d(g)   (flux.f90:751-928)
    for d, name in enumerate(("VX", "VY", "VZ")):
        rows = []
        for pt in interior:
            row = []
            for f, c in zip(fams, cb):
                degs = list(f)
                val = 1.0
                for e in range(3):
                    val = val * (dL(degs[e], pt[e]) if e == d else L(degs[e], pt[e]))
                row.append(0.25 * c * w3[len(rows)] * val)
            rows.append(row)
        T[name] = rows
    # surface quadrature: +-0.25*cbasis(b)*w2d(p)*phi_b(face point)  (flux.f90:958-978)
    for k in ("xp", "xm", "yp", "ym", "zp", "zm"):
        sgn = 1.0 if k.endswith("p") else -1.0
        T["S" + k.upper()] = [[sgn * 0.25 * c * w2[p] * v for c, v in zip(cb, T[k.upper()][p])] for p in range(len(w2))]
    # source projection: 0.125*cbasis(b)*wgt3d(g)*phi_b(g)   (sources.f90:74-78)
    T["SRC"] = [[0.125 * c * (w3[g] * v) for c, v in zip(cb, T["INT"][g])] for g in range(len(w3))]
    T["CB"] = cb
    T["W2"] = w2
    T["W3"] = w3
    return T


def _lit(v: float) -> str:
    if v == 0.0:
        return "0.0"
    return v.hex()


def emit(path: str) -> None:
    out = ["// Generated by gen_tables.py -- do not edit.  Legendre basis and Gauss",
           "// quadrature tables of the supported (nbasis, iquad) pairs as compile-time",
           "// constants (values bit-identical to the reference's table setup,",
           "// basis_funcs.f90:265-627 and initialize.f90:126-220).",
           "#pragma once", "", "namespace hermes_tab {", "",
           "template <int NB, int NQD> struct Tab;", ""]
    for (nb, iq) in FAMILIES:
        T = tables(nb, iq)
        nf, npg = iq * iq, iq ** 3
        out.append(f"template <> struct Tab<{nb}, {iq}> {{")
        out.append(f"    static constexpr int NB = {nb}, NQD = {iq}, NF = {nf}, NPG = {npg}, NPGE = {6 * nf};")
        degs = ", ".join("{" + ", ".join(str(d) for d in fam) + "}" for fam in FAMILIES[(nb, iq)])
        out.append(f"    // Legendre degree of basis function b along axis a (x, y, z)")
        out.append(f"    static constexpr int DEG(int b, int a) {{ const int t[{nb}][3] = {{{degs}}}; return t[b][a]; }}")
        for name, rows in T.items():
            if name in ("CB", "W2", "W3"):
                vals = ", ".join(_lit(v) for v in rows)
                out.append(f"    static constexpr double {name}(int i) {{ const double t[{len(rows)}] = {{{vals}}}; return t[i]; }}")
                continue
            nr = len(rows)
            body = ", ".join("{" + ", ".join(_lit(v) for v in r) + "}" for r in rows)
            out.append(f"    static constexpr double {name}(int r, int b) {{ const double t[{nr}][{nb}] = {{{body}}}; return t[r][b]; }}")
        out.append("};")
        out.append("")
    out.append("}  // namespace hermes_tab")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    emit(os.path.join(os.path.dirname(os.path.abspath(__file__)), "dg_tables_gen.cuh"))

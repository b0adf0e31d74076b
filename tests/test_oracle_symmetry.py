"""The oracle's right-hand side commutes with the exchange of the x and y
axes on a square periodic grid (swap the cell indices, the momenta m_x <-> m_y,
the stresses P_xx <-> P_yy and P_xz <-> P_yz, and the basis functions, x <-> y
in every Legendre product) and with the reflection x -> -x (cells in reverse
order, m_x, P_xy, P_xz and the basis functions odd in x negated): the
right-hand side comes out transformed the same way, to rounding.  Every
direction-specific table, flux and index of the restatement, and the
left/right roles of every face, are exercised against their mirrors."""
import numpy as np
import pytest

from hermeshd_gb300 import config, ic

RH, MX, MY, MZ, EN, PXX, PYY, PZZ, PXY, PXZ, PYZ = range(11)
VAR_SWAP = [RH, MY, MX, MZ, EN, PYY, PXX, PZZ, PXY, PYZ, PXZ]


def basis_swap(kindex, nb):
    """0-based permutation of the coefficients under x <-> y."""
    names = ["kx", "ky", "kz", "kyz", "kzx", "kxy", "kxyz", "kxx", "kyy", "kzz"]
    k = {n: int(kindex[i]) - 1 for i, n in enumerate(names)}
    perm = list(range(nb))
    for a, b in (("kx", "ky"), ("kyz", "kzx"), ("kxx", "kyy")):
        if k[a] < nb and k[b] < nb:
            perm[k[a]], perm[k[b]] = k[b], k[a]
    return perm


def swap(Q, perm):
    S = np.transpose(Q, (1, 0, 2, 3, 4))       # (x, y) cell indices exchanged
    S = S[:, :, :, VAR_SWAP, :]
    S = S[:, :, :, :, perm]
    return np.asfortranarray(S)


@pytest.mark.parametrize("nb,iq", [(4, 2), (8, 2), (10, 3)])
@pytest.mark.parametrize("ivis,ihllc", [(0, 1), (1, 2), (1, 0), (2, 1)])
def test_rhs_commutes_with_the_xy_exchange(nb, iq, ivis, ihllc):
    import oracle as O
    cfg = config.Config(nx=5, ny=5, nz=2, nbasis=nb, iquad=iq, ivis=ivis, ihllc=ihllc, coll=1.3, colvis=0.7,
                        lx=2.0, ly=2.0, lz=1.0)
    orc = O.Oracle(cfg)
    perm = basis_swap(orc.kindex(), nb)
    Q = ic.random_smooth(cfg, seed=nb + 10 * ivis + ihllc, amp=0.05, stress_amp=0.02)
    if ivis == 2:
        Q = ic.ten_moment_stress(cfg, Q, p=1.0, amp=0.01, seed=1)
    R = orc.rhs(np.asfortranarray(Q), limit=False)
    Rs = orc.rhs(swap(Q, perm), limit=False)
    scale = np.abs(R).max()
    assert scale > 0
    assert np.allclose(Rs, swap(R, perm), rtol=0, atol=1e-12 * scale), float(np.abs(Rs - swap(R, perm)).max() / scale)


def reflect_x(Q, kindex, nb):
    """x -> -x: the cell order reversed in x, m_x, P_xy, P_xz negated, and the
    basis functions odd in x (x, zx, xy, xyz) negated."""
    names = ["kx", "ky", "kz", "kyz", "kzx", "kxy", "kxyz", "kxx", "kyy", "kzz"]
    k = {n: int(kindex[i]) - 1 for i, n in enumerate(names)}
    sb = np.ones(nb)
    for n in ("kx", "kzx", "kxy", "kxyz"):
        if k[n] < nb:
            sb[k[n]] = -1.0
    sv = np.ones(11)
    sv[[MX, PXY, PXZ]] = -1.0
    S = Q[::-1, :, :, :, :] * sv[None, None, None, :, None] * sb[None, None, None, None, :]
    return np.asfortranarray(S)


@pytest.mark.parametrize("nb,iq", [(4, 2), (8, 2), (10, 3)])
@pytest.mark.parametrize("ivis,ihllc", [(0, 1), (1, 2), (1, 0), (2, 1)])
def test_rhs_commutes_with_the_x_reflection(nb, iq, ivis, ihllc):
    import oracle as O
    cfg = config.Config(nx=6, ny=4, nz=2, nbasis=nb, iquad=iq, ivis=ivis, ihllc=ihllc, coll=1.3, colvis=0.7,
                        lx=2.4, ly=1.6, lz=1.0)
    orc = O.Oracle(cfg)
    kin = orc.kindex()
    Q = ic.random_smooth(cfg, seed=2 * nb + ivis + 7 * ihllc, amp=0.05, stress_amp=0.02)
    if ivis == 2:
        Q = ic.ten_moment_stress(cfg, Q, p=1.0, amp=0.01, seed=2)
    R = orc.rhs(np.asfortranarray(Q), limit=False)
    Rr = orc.rhs(reflect_x(Q, kin, nb), limit=False)
    scale = np.abs(R).max()
    assert np.allclose(Rr, reflect_x(R, kin, nb), rtol=0, atol=1e-12 * scale), \
        float(np.abs(Rr - reflect_x(R, kin, nb)).max() / scale)


def exchange_xz(Q, kindex, nb):
    """x <-> z: cell indices, m_x <-> m_z, P_xx <-> P_zz, P_xy <-> P_yz, and the
    basis functions x <-> z, xy <-> yz, xx <-> zz."""
    names = ["kx", "ky", "kz", "kyz", "kzx", "kxy", "kxyz", "kxx", "kyy", "kzz"]
    k = {n: int(kindex[i]) - 1 for i, n in enumerate(names)}
    perm = list(range(nb))
    for a, b in (("kx", "kz"), ("kxy", "kyz"), ("kxx", "kzz")):
        if k[a] < nb and k[b] < nb:
            perm[k[a]], perm[k[b]] = k[b], k[a]
    var = [RH, MZ, MY, MX, EN, PZZ, PYY, PXX, PYZ, PXZ, PXY]
    S = np.transpose(Q, (2, 1, 0, 3, 4))[:, :, :, var, :][:, :, :, :, perm]
    return np.asfortranarray(S)


@pytest.mark.parametrize("nb,iq", [(4, 2), (8, 2), (10, 3)])
@pytest.mark.parametrize("ivis,ihllc", [(1, 1), (2, 2)])
def test_rhs_commutes_with_the_xz_exchange(nb, iq, ivis, ihllc):
    import oracle as O
    cfg = config.Config(nx=4, ny=3, nz=4, nbasis=nb, iquad=iq, ivis=ivis, ihllc=ihllc, coll=1.3, colvis=0.7,
                        lx=1.6, ly=1.2, lz=1.6)
    orc = O.Oracle(cfg)
    kin = orc.kindex()
    Q = ic.random_smooth(cfg, seed=3 * nb + ivis, amp=0.05, stress_amp=0.02)
    if ivis == 2:
        Q = ic.ten_moment_stress(cfg, Q, p=1.0, amp=0.01, seed=3)
    R = orc.rhs(np.asfortranarray(Q), limit=False)
    Rx = orc.rhs(exchange_xz(Q, kin, nb), limit=False)
    scale = np.abs(R).max()
    assert np.allclose(Rx, exchange_xz(R, kin, nb), rtol=0, atol=1e-12 * scale), \
        float(np.abs(Rx - exchange_xz(R, kin, nb)).max() / scale)

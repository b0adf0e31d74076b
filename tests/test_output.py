"""Derived fields of the VTK output (output.f90:14-317): the numpy
restatement's tables and closed-form values on the CPU, the .vtr writer, and
the CUDA kernel against the restatement on the GPU.

Tolerance of the CUDA path (float32 output of FP64 arithmetic): 4 float32
ulps relative to each variable's largest magnitude."""
import base64
import struct
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from hermeshd_gb300 import config, ic


def _decode(text):
    raw = base64.b64decode(text.strip())
    n = struct.unpack("<I", raw[:4])[0]
    return np.frombuffer(raw[4:4 + n], dtype="<f4")


def test_vtk_tables_at_cell_centre_and_subpoints():
    import derived_ref as D
    cfg = config.Config(nx=2, ny=2, nz=2, nbasis=10, iquad=3)
    bf, dx, dy = D.vtk_tables(cfg, 1)
    assert np.array_equal(bf[0], [1, 0, 0, 0, 0, 0, 0, -0.5, -0.5, -0.5])
    assert np.array_equal(dx[0], [0, 1, 0, 0, 0, 0, 0, 0, 0, 0])
    bf, dx, dy = D.vtk_tables(config.Config(nx=2, ny=2, nz=2, nbasis=8, iquad=2), 2)
    # igrid = 4*ix + 2*iy + iz with coordinates -1/2, 1/2; basis {1,x,y,z,yz,zx,xy,xyz}
    g = 4 * 1 + 2 * 0 + 1
    x, y, z = 0.5, -0.5, 0.5
    assert np.allclose(bf[g], [1, x, y, z, y * z, z * x, x * y, x * y * z], rtol=0, atol=0)
    assert np.allclose(dx[g], [0, 1, 0, 0, 0, z, y, y * z], rtol=0, atol=0)


def test_uniform_state_values():
    import derived_ref as D
    cfg = config.Config(nx=3, ny=2, nz=1, nbasis=4, iquad=2, aindex=1.4)
    Q = ic.equilibrium(cfg)
    rho, vx, p = 2.0, 0.3, 1.5
    Q[:, :, :, 0, 0] = rho
    Q[:, :, :, 1, 0] = rho * vx
    Q[:, :, :, 4, 0] = p / 0.4 + 0.5 * rho * vx * vx
    out = D.derived(cfg, Q, 1, n0=10.0, v0=2.0, te0=3.0, eV_per_K=0.5)
    assert np.allclose(out[0], rho * 10.0) and np.allclose(out[1], np.log10(20.0))
    assert np.allclose(out[2], 2.0 * vx) and np.allclose(out[5], p * 3.0 / rho / 0.5)
    assert np.allclose(out[9], p) and np.allclose(out[13], 0.0)


def test_vtr_writer(tmp_path):
    from hermeshd_gb300.output import write_vtr
    cfg = config.Config(nx=3, ny=2, nz=1, nbasis=4, iquad=2, lx=3.0, ly=2.0, lz=1.0)
    d = np.arange(6, dtype=np.float32).reshape(1, 2, 3)
    v = np.stack([d, d + 10, d + 20])
    p = write_vtr(str(tmp_path / "a.vtr"), cfg, {"Density": d, "Velocity": v}, nvtk=1)
    root = ET.parse(p).getroot()
    assert root.attrib["type"] == "RectilinearGrid"
    arrays = {a.attrib["Name"]: a for a in root.iter("DataArray")}
    assert np.allclose(_decode(arrays["X"].text), [-1.5, -0.5, 0.5, 1.5])
    assert np.array_equal(_decode(arrays["Density"].text), d.reshape(-1))
    vv = _decode(arrays["Velocity"].text).reshape(-1, 3)
    assert np.array_equal(vv[:, 1], (d + 10).reshape(-1)) and arrays["Velocity"].attrib["NumberOfComponents"] == "3"


CASES = [
    (config.Config(nx=6, ny=5, nz=4, nbasis=4, iquad=2), 1),
    (config.Config(nx=5, ny=4, nz=3, nbasis=8, iquad=2, ivis=1, coll=1.0, colvis=1.0), 2),
    (config.Config(nx=6, ny=6, nz=1, nbasis=10, iquad=3), 3),
    (config.Config(nx=4, ny=3, nz=2, nbasis=10, iquad=3, precision="fp32"), 2),
]


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(len(CASES)))
def test_cuda_derived_fields_match_restatement(k):
    import derived_ref as D
    from hermeshd_gb300.config import Units
    from hermeshd_gb300.output import VARIABLES, derived
    from hermeshd_gb300.solver import Solver
    cfg, nvtk = CASES[k]
    Q = ic.random_smooth(cfg, seed=k, amp=0.1, stress_amp=0.05)
    s = Solver(cfg)
    q = s.from_numpy(Q)
    u = Units()
    arr, names = derived(s, q, VARIABLES, nvtk, u)
    assert list(names) == list(VARIABLES)
    Qin = s.to_numpy(q)     # the FP32 path's own input, widened
    ref = D.derived(cfg, Qin, nvtk, n0=u.n0, v0=1.0, t0=1.0, te0=u.te0, eV_per_K=u.eV_per_K)
    got = arr.cpu().numpy().astype(np.float64)
    for v in range(len(VARIABLES)):
        scale = np.abs(ref[v]).max()
        assert np.abs(got[v] - ref[v]).max() <= 4 * 2.0 ** -23 * scale + 1e-30, VARIABLES[v]


@pytest.mark.gpu
def test_output_vtk_file(tmp_path):
    from hermeshd_gb300.output import derived, output_vtk
    from hermeshd_gb300.solver import Solver
    cfg = config.isentropic_vortex_2d(n=16)
    s = Solver(cfg)
    q = s.from_numpy(ic.isentropic_vortex(cfg))
    p = output_vtk(s, q, nout=3, outdir=str(tmp_path))
    assert p.endswith("perseus_p0000_t0003.vtr")
    arrays = {a.attrib["Name"]: a for a in ET.parse(p).getroot().iter("DataArray")}
    assert set(arrays) == {"X", "Y", "Z", "Density", "Velocity", "Temperature", "Pressure"}
    arr, names = derived(s, q, ("Density",))
    assert np.array_equal(_decode(arrays["Density"].text), arr.cpu().numpy().reshape(-1))

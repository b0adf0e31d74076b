"""Checkpoint files in the format of writeQ / readQ (initialize.f90:474-565):
exact FP64 round trip, the record layout, Fortran list-directed input forms
the reference's own files may contain, error reporting, file names and the
odd/even rotation (hermeshd.f90:248-252), restart checks.  Host only."""
import os

import numpy as np
import pytest

from hermeshd_gb300 import checkpoint, config
from hermeshd_gb300._lib import HermesError


def _state(cfg, seed=0):
    rng = np.random.default_rng(seed)
    Q = np.asfortranarray(rng.standard_normal(cfg.shape_f))
    Q.flat[0] = -0.0
    Q.flat[1] = 5e-324          # smallest subnormal
    Q.flat[2] = 1.7976931348623157e308
    Q.flat[3] = -1.0 / 3.0
    return Q


def test_round_trip_is_exact(hermes_lib, tmp_path):
    cfg = config.Config(nx=7, ny=3, nz=2, nbasis=4, iquad=2)
    Q = _state(cfg)
    p = str(tmp_path / "q.dat")
    checkpoint.write(p, Q, 1.25, 3.0e-3, 17, (1, 1, 1))
    R, t, dt, nout, md = checkpoint.read(p, cfg)
    assert np.array_equal(R.view(np.uint64), Q.view(np.uint64))   # bit for bit, signed zero included
    assert (t, dt, nout, md) == (1.25, 3.0e-3, 17, (1, 1, 1))


def test_record_layout(hermes_lib, tmp_path):
    cfg = config.Config(nx=5, ny=2, nz=3, nbasis=8, iquad=2)
    Q = _state(cfg, 1)
    p = str(tmp_path / "q.dat")
    checkpoint.write(p, Q, 0.5, 0.01, 3, (2, 1, 1))
    lines = open(p).read().splitlines()
    assert len(lines) == cfg.nbasis * 11 * cfg.nz * cfg.ny + 1
    r = 0
    for b in range(cfg.nbasis):
        for v in range(11):
            for k in range(cfg.nz):
                for j in range(cfg.ny):
                    vals = [float(x) for x in lines[r].split()]
                    assert vals == list(Q[:, j, k, v, b])
                    r += 1
    last = lines[-1].split()
    assert [float(last[0]), float(last[1])] == [0.5, 0.01] and last[2:] == ["3", "2", "1", "1"]


def test_reads_list_directed_forms(hermes_lib, tmp_path):
    """Spacing and digits of a REAL*4 list-directed write, repeat counts, null
    values, commas, D exponents, sign-only exponents, rows continued on the
    next line, blank lines and a slash."""
    cfg = config.Config(nx=4, ny=1, nz=1, nbasis=4, iquad=2)
    rows = 4 * 11
    want = np.zeros(cfg.shape_f, order="F")
    text = []
    for r in range(rows):
        b, v = divmod(r, 11)
        if r == 0:
            text.append("   1.00000000       2.50000000E-02  -3.00000000       4.00000000    ")
            want[:, 0, 0, v, b] = [1.0, 2.5e-2, -3.0, 4.0]
        elif r == 1:
            text.append(" 4*0.500000000")
            want[:, 0, 0, v, b] = 0.5
        elif r == 2:
            text.append("1.5D+00, 2.0d-1,3.0-1 ,  4")
            want[:, 0, 0, v, b] = [1.5, 0.2, 0.3, 4.0]
        elif r == 3:
            text.append("   7.0   8.0")
            text.append("")
            text.append("   9.0  10.0   99.0")      # the rest of the record is skipped
            want[:, 0, 0, v, b] = [7.0, 8.0, 9.0, 10.0]
        elif r == 4:
            text.append("1.0 /")                     # a slash leaves the rest unchanged (zero here)
            want[:, 0, 0, v, b] = [1.0, 0.0, 0.0, 0.0]
        elif r == 5:
            text.append("2*, 3.0 4.0")               # two null values
            want[:, 0, 0, v, b] = [0.0, 0.0, 3.0, 4.0]
        else:
            text.append(" ".join(repr(float(r + i)) for i in range(4)))
            want[:, 0, 0, v, b] = [float(r + i) for i in range(4)]
    text.append("   2.00000003E-02   1.00000005E-03          12           1           1           1")
    p = tmp_path / "ref.dat"
    p.write_text("\n".join(text) + "\n")
    Q, t, dt, nout, md = checkpoint.read(str(p), cfg)
    assert np.array_equal(Q, want)
    assert (t, dt, nout, md) == (2.00000003e-2, 1.00000005e-3, 12, (1, 1, 1))


def test_short_or_bad_file_is_an_error(hermes_lib, tmp_path):
    cfg = config.Config(nx=4, ny=2, nz=1, nbasis=4, iquad=2)
    p = str(tmp_path / "q.dat")
    checkpoint.write(p, _state(cfg), 0.0, 0.1, 0)
    lines = open(p).read().splitlines()
    short = tmp_path / "short.dat"
    short.write_text("\n".join(lines[:10]) + "\n")
    with pytest.raises(HermesError, match="file ends"):
        checkpoint.read(str(short), cfg)
    bad = tmp_path / "bad.dat"
    bad.write_text("\n".join(["1.0 2.0 x3 4.0"] + lines[1:]) + "\n")
    with pytest.raises(HermesError, match="bad value 'x3'"):
        checkpoint.read(str(bad), cfg)
    with pytest.raises(HermesError, match="cannot open"):
        checkpoint.read(str(tmp_path / "missing.dat"), cfg)


def test_names_rotation_and_restart(hermes_lib, tmp_path):
    assert checkpoint.checkpoint_name("Qout", 0, 1) == "Qout_p0000_d0001.dat"
    assert checkpoint.checkpoint_name("Qout", 12, 2) == "Qout_p0012_d0002.dat"
    assert [checkpoint.odd_even_dump(n) for n in (1, 2, 3, 4)] == [1, 2, 1, 2]
    cfg = config.Config(nx=4, ny=2, nz=1, nbasis=4, iquad=2)
    d = str(tmp_path / "data")
    Q = np.asfortranarray(np.random.default_rng(3).standard_normal(cfg.shape_f))
    for nout in (1, 2, 3):
        checkpoint.write_dump(d, Q * nout, t=0.1 * nout, dt=0.01, nout=nout)
    assert sorted(os.listdir(d)) == ["Qout_p0000_d0001.dat", "Qout_p0000_d0002.dat"]
    # dump 1 holds nout = 3 at t = 0.3: dtout = t/(nout-1) = 0.15
    R, t, dt, nout = checkpoint.restart(d, cfg, dump=1, dtout=0.15, resuming=True)
    assert np.array_equal(R, Q * 3) and (t, dt, nout) == (0.1 * 3, 0.01, 3)
    R, t, dt, nout = checkpoint.restart(d, cfg, dump=1, dtout=0.05, resuming=False)
    assert (t, dt, nout) == (0.0, 0.0, 0)
    with pytest.raises(HermesError, match="dtout"):
        checkpoint.restart(d, cfg, dump=1, dtout=5.0, resuming=True)
    with pytest.raises(HermesError, match="mpi"):
        checkpoint.restart(d, cfg, dump=1, dtout=0.15, resuming=True, mpi_dims=(2, 1, 1))


@pytest.mark.gpu
def test_front_end_writes_and_resumes(tmp_path):
    """Hermeshd.generate_output writes odd/even checkpoints when iwrite = 1;
    setup with iread and resuming continues from the file's state and clock."""
    from hermeshd_gb300.hermeshd import Hermeshd
    cfg = config.sod_1d(nx=64).replace(tf=0.02, ntout=4)
    h = Hermeshd()
    h.configure(cfg, icid=3, iwrite=1, datadir=str(tmp_path))
    Q = np.zeros(cfg.shape_f, order="F")
    Q1, Q2 = np.zeros_like(Q), np.zeros_like(Q)
    t, dt, t1, ts, dtout, nout = (np.array(0.0), np.array(0.0), np.array(0.0), np.array(0.0), np.array(0.0),
                                  np.array(0))
    h.setup(Q, t, dt, t1, ts, dtout, nout)
    saved = {}
    while float(t) < cfg.tf:
        h.step(Q, Q1, Q2, t, dt)
        n0 = int(nout)
        h.generate_output(Q, t, dt, t1, dtout, nout)
        if int(nout) != n0:
            saved[int(nout)] = (Q.copy(), float(t), float(dt))
    last = max(saved)
    dump = checkpoint.odd_even_dump(last)
    R, tr, dtr, nr, _ = checkpoint.read(str(tmp_path / checkpoint.checkpoint_name("Qout", 0, dump)), cfg)
    assert np.array_equal(R, saved[last][0]) and (tr, dtr, nr) == (saved[last][1], saved[last][2], last)
    h.cleanup(ts)
    h2 = Hermeshd()
    h2.configure(cfg, icid=3, iread=dump, resuming=True, datadir=str(tmp_path))
    Qb = np.zeros_like(Q)
    tb, dtb, t1b, tsb, dtoutb, noutb = (np.array(0.0), np.array(0.0), np.array(0.0), np.array(0.0), np.array(0.0),
                                        np.array(0))
    h2.setup(Qb, tb, dtb, t1b, tsb, dtoutb, noutb)
    assert np.array_equal(Qb, saved[last][0]) and float(tb) == saved[last][1] and int(noutb) == last
    h2.cleanup(tsb)

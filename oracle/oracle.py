"""ctypes wrapper of the CPU FP64 oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this module; the product package never does.  The oracle restates the
reference's step path in C (hermes_oracle.c); arrays are the reference's
Fortran-ordered Q(nx,ny,nz,nQ,nbasis) float64.

Parity pinning: the reference cannot be compiled here and ships no golden
vectors; its routines executed from their Fortran source
(tests/golden/fortran_subset.py, tests/golden/make_reference_vectors.py)
produce this oracle's tables, limiter, face fluxes, right-hand sides and steps
bit for bit on the cases of tests/golden/reference/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "libhermes_oracle.so")
# the same source built for timing only (host-tuned, FMA contraction on):
# the CPU baseline's clock, never the checker (its roundings differ)
LIB_TIMING = os.path.join(HERE, "build", "libhermes_oracle_timing.so")


class OrcParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("nbasis", C.c_int), ("iquad", C.c_int),
        ("ivis", C.c_int), ("ieos", C.c_int), ("ihllc", C.c_int), ("iorder", C.c_int),
        ("bc", C.c_int * 6),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("aindex", C.c_double), ("rh_floor", C.c_double), ("T_floor", C.c_double),
        ("coll", C.c_double), ("colvis", C.c_double), ("cflm", C.c_double),
        ("P_1", C.c_double), ("P_base", C.c_double), ("rh_mult", C.c_double),
        ("llns", C.c_int), ("pad_", C.c_int),
        ("eta_sd", C.c_double), ("zeta_sd", C.c_double), ("seed", C.c_ulonglong),
        ("body_force", C.c_double),
        ("inflow_u", C.c_double), ("inflow_rho", C.c_double), ("inflow_p", C.c_double),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle's parity and timing builds with its Makefile (gcc, OpenMP)."""
    src = max(os.path.getmtime(os.path.join(HERE, f)) for f in ("hermes_oracle.c", "hermes_oracle.h", "philox_ref.h",
                                                                  "Makefile"))
    if force or any(not os.path.exists(p) or os.path.getmtime(p) < src for p in (LIB, LIB_TIMING)):
        subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    return LIB


def timing_flags() -> str:
    """The compiler flags of the timing build on this host."""
    return subprocess.run(["make", "-s", "-C", HERE, "timing_flags"], capture_output=True, text=True).stdout.strip()


_libs = {}


def lib(timing: bool = False):
    """The parity build (the checker), or with timing=True the host-tuned
    build that bench.py times as the CPU baseline."""
    L = _libs.get(timing)
    if L is None:
        build()
        L = C.CDLL(LIB_TIMING if timing else LIB)
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(OrcParams)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_qsize.restype = C.c_long
        L.orc_qsize.argtypes = [C.c_void_p]
        L.orc_cflm.restype = C.c_double
        L.orc_cflm.argtypes = [C.c_void_p]
        L.orc_get_table.restype = C.c_int
        L.orc_get_table.argtypes = [C.c_void_p, C.c_char_p, np.ctypeslib.ndpointer(dtype=np.float64), C.c_int]
        L.orc_get_kindex.restype = C.c_int
        L.orc_get_kindex.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(dtype=np.int32)]
        L.orc_limiter.argtypes = [C.c_void_p, dp]
        L.orc_prep_and_rhs.argtypes = [C.c_void_p, dp, dp]
        L.orc_rhs_nolimit.argtypes = [C.c_void_p, dp, dp]
        L.orc_euler_step.argtypes = [C.c_void_p, dp, dp, C.c_double]
        L.orc_get_min_dt.restype = C.c_double
        L.orc_get_min_dt.argtypes = [C.c_void_p, dp]
        L.orc_step.argtypes = [C.c_void_p, dp, dp, dp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_advance.restype = C.c_int
        L.orc_advance.argtypes = [C.c_void_p, dp, dp, dp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int]
        L.orc_advance_fixed_dt.argtypes = [C.c_void_p, dp, dp, dp, C.c_double, C.c_int]
        L.orc_set_noise_counter.argtypes = [C.c_void_p, C.c_ulonglong]
        L.orc_get_timers.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(dtype=np.float64)]
        L.orc_reset_timers.argtypes = [C.c_void_p]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_num_threads.argtypes = [C.c_int]
        L.orc_noise_sample.argtypes = [C.c_ulonglong, C.c_ulonglong, C.c_uint, C.c_uint, C.c_ulonglong, C.c_uint,
                                       C.c_double, C.c_double, np.ctypeslib.ndpointer(dtype=np.float64),
                                       np.ctypeslib.ndpointer(dtype=np.float64)]
        u32p = np.ctypeslib.ndpointer(dtype=np.uint32)
        L.orc_philox4x32_10.argtypes = [u32p, C.c_uint32, C.c_uint32, u32p]
        L.orc_test_basis.restype = C.c_double
        L.orc_test_basis.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _libs[timing] = L
    return L


def params_from_config(cfg) -> OrcParams:
    p = OrcParams()
    p.nx, p.ny, p.nz = cfg.nx, cfg.ny, cfg.nz
    p.nbasis, p.iquad = cfg.nbasis, cfg.iquad
    p.ivis, p.ieos, p.ihllc, p.iorder = cfg.ivis, cfg.ieos, int(cfg.ihllc), cfg.iorder
    for i, b in enumerate(cfg.bc):
        p.bc[i] = b
    p.lx, p.ly, p.lz = cfg.lx, cfg.ly, cfg.lz
    p.aindex, p.rh_floor, p.T_floor = cfg.aindex, cfg.rh_floor, cfg.T_floor
    p.coll, p.colvis, p.cflm = cfg.coll, cfg.colvis, cfg.cflm
    p.P_1, p.P_base, p.rh_mult = cfg.P_1, cfg.P_base, cfg.rh_mult
    p.llns = int(cfg.llns)
    p.eta_sd, p.zeta_sd, p.seed = cfg.eta_sd, cfg.zeta_sd, cfg.seed
    p.body_force = cfg.body_force
    p.inflow_u, p.inflow_rho, p.inflow_p = cfg.inflow_u, cfg.inflow_rho, cfg.inflow_pressure
    return p


class Oracle:
    """One oracle context for one Config (timing=True: the host-tuned build,
    for the CPU baseline's clock only)."""

    def __init__(self, cfg, timing: bool = False):
        cfg.validate(oracle=True)
        self.cfg = cfg
        self.L = lib(timing)
        self._p = params_from_config(cfg)
        self.h = self.L.orc_create(C.byref(self._p))
        if not self.h:
            raise MemoryError("orc_create failed")

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def _arr(self, Q):
        if not (isinstance(Q, np.ndarray) and Q.dtype == np.float64 and Q.flags.f_contiguous and Q.shape == self.cfg.shape_f):
            raise ValueError("expected float64 Fortran-ordered array of shape %s" % (self.cfg.shape_f,))
        return Q

    def new(self):
        return np.zeros(self.cfg.shape_f, dtype=np.float64, order="F")

    def table(self, name):
        out = np.zeros(200 * 31, dtype=np.float64)
        n = self.L.orc_get_table(self.h, name.encode(), out, out.size)
        if n < 0:
            raise KeyError(name)
        if name in ("cbasis", "wgt3d", "wgt2d"):
            return out[:n].copy()
        return out[:n].reshape(-1, 30).copy()

    def kindex(self):
        out = np.zeros(29, dtype=np.int32)
        self.L.orc_get_kindex(self.h, out)
        return out

    @property
    def cflm(self):
        return self.L.orc_cflm(self.h)

    def limiter(self, Q):
        self.L.orc_limiter(self.h, self._arr(Q))

    def rhs(self, Q, limit=True):
        """glflux - source for the state Q (limited in place first if limit)."""
        out = self.new()
        if limit:
            self.L.orc_prep_and_rhs(self.h, self._arr(Q), out)
        else:
            self.L.orc_rhs_nolimit(self.h, self._arr(Q), out)
        return out

    def euler_step(self, Qin, dt):
        out = self.new()
        self.L.orc_euler_step(self.h, self._arr(Qin), out, dt)
        return out

    def get_min_dt(self, Q):
        return self.L.orc_get_min_dt(self.h, self._arr(Q))

    def step(self, Q, Q1, Q2, t, dt):
        tt, dd = C.c_double(t), C.c_double(dt)
        self.L.orc_step(self.h, self._arr(Q), self._arr(Q1), self._arr(Q2), C.byref(tt), C.byref(dd))
        return tt.value, dd.value

    def advance(self, Q, nsteps, t=0.0, Q1=None, Q2=None):
        Q1 = self.new() if Q1 is None else Q1
        Q2 = self.new() if Q2 is None else Q2
        tt, dd = C.c_double(t), C.c_double(0.0)
        n = self.L.orc_advance(self.h, self._arr(Q), Q1, Q2, C.byref(tt), C.byref(dd), nsteps)
        if n < 0:
            raise FloatingPointError("oracle: NaN cell average at step %d" % (-n))
        return tt.value, dd.value

    def advance_fixed_dt(self, Q, dt, nsteps, Q1=None, Q2=None):
        Q1 = self.new() if Q1 is None else Q1
        Q2 = self.new() if Q2 is None else Q2
        self.L.orc_advance_fixed_dt(self.h, self._arr(Q), Q1, Q2, dt, nsteps)

    def set_noise_counter(self, step):
        self.L.orc_set_noise_counter(self.h, step)

    def timers(self):
        out = np.zeros(6)
        self.L.orc_get_timers(self.h, out)
        return dict(zip(("limiter", "faces", "volume", "surface", "source", "update"), out))

    def reset_timers(self):
        self.L.orc_reset_timers(self.h)

    def test_basis(self):
        a, b = C.c_double(), C.c_double()
        self.L.orc_test_basis(self.h, C.byref(a), C.byref(b))
        return a.value, b.value


def num_threads():
    return lib().orc_num_threads()


def set_num_threads(n):
    lib().orc_set_num_threads(n)


def noise_sample(seed, step, stage, kind, site, pt, eta=1.0, zeta=0.0):
    """(6 normals {xx, yy, zz, xy, xz, yz}, stress {xx,yy,zz,xy,xz,yz}) of one
    point of one flux call."""
    G = np.zeros(6)
    S = np.zeros(6)
    lib().orc_noise_sample(seed, step, stage, kind, site, pt, eta, zeta, G, S)
    return G, S


def philox4x32_10(ctr, key):
    """One Philox-4x32-10 block: ctr = 4 words, key = 2 words -> 4 words."""
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(c, int(key[0]), int(key[1]), out)
    return [int(x) for x in out]

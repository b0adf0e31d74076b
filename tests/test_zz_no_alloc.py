"""hermes_rhs_noalloc: the right-hand side without a context or any device
allocation, for callers that cannot allocate device memory when they need
it (a host framework that owns all device memory, or a time loop that must
not pay cudaMalloc's synchronisation).  Its face-flux scratch is a static
device array shared by every call.

Checked through the C ABI against the context path (hermes_rhs, which
allocates its scratch in hermes_create), on two calls in a row, at the
tolerance of the right-hand-side parity tests.  With the stochastic stress
on, every call draws the realisation of step 0, stage 0: the reference is
then hermes_rhs on a fresh context (its noise counter at step 0), whose
staged draws are the same Philox numbers.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from hermeshd_gb300 import _lib, config, ic
from helpers import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _noalloc(L, cfg, q, out, limit=0):
    import torch
    err = C.create_string_buffer(256)
    rc = L.hermes_rhs_noalloc(C.byref(_lib.to_c(cfg)), C.c_void_p(q.data_ptr()), C.c_void_p(out.data_ptr()), limit,
                              C.c_void_p(torch.cuda.current_stream().cuda_stream), err, 256)
    return rc, err.value.decode()


@pytest.mark.parametrize("cfg", [
    config.isentropic_vortex_2d(n=24),
    config.Config(nx=6, ny=5, nz=4, nbasis=4, iquad=2, ivis=1, coll=2.0, colvis=1.0, xlobc="wall", xhibc="noslip",
                  precision="fp32"),
    config.fh_box(8, precision="fp64", seed=5),
    config.fh_box(8, precision="fp32", seed=5),
], ids=["vortex24_nb10_f64", "box_nb4_f32_walls", "fh8_noise_f64", "fh8_noise_f32"])
def test_noalloc_rhs_matches_context_rhs_twice(cfg):
    import torch
    from hermeshd_gb300.solver import Solver
    L = _lib.lib()
    tol = TOL if cfg.precision == "fp64" else 1e-6
    for call, seed in enumerate((3, 4)):
        s = Solver(cfg)          # a fresh context: noise counter at step 0
        Q = ic.random_smooth(cfg, seed=seed, amp=0.05, stress_amp=0.01)
        q = s.from_numpy(Q)
        ref = s.rhs(q.clone(), limit=True)
        qn = q.clone()
        out = torch.full_like(q, float("nan"))
        rc, msg = _noalloc(L, cfg, qn, out, limit=1)
        assert rc == 0, msg
        torch.cuda.synchronize()
        err = rel_l2(out.double().cpu().numpy(), ref.double().cpu().numpy())
        assert err <= tol, f"call {call}: rel L2 {err:.3e}"
        s.close()


def test_noalloc_rejects_oversize_grid():
    import torch
    L = _lib.lib()
    cfg = config.Config(nx=256, ny=256, nz=4, nbasis=10, iquad=3)     # ~0.3 GB of face fluxes
    q = torch.zeros(1, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc, msg = _noalloc(L, cfg, q, out)
    assert rc == 2 and "static maximum" in msg

"""Generate the golden fixtures of tests/golden/ from the FP64 oracle.

The reference (Fortran 90 + MPI + MKL) cannot be built or run here and its
tests store no vectors, so these fixtures are the oracle's outputs on small
seeded cases -- a frozen record of the reference's algorithm as restated in
oracle/hermes_oracle.c.  tests/test_golden.py checks that the oracle still
reproduces them and that the CUDA path matches them.

Each case stores: the input state Q0 (Fortran order Q(nx,ny,nz,nQ,nbasis)),
the right-hand side of Q0 (limiter applied), the state after `steps` steps
with the time and last time step, and the Config fields.

Run from the repository root:  python tests/golden/make_golden.py [case ...]
(no arguments: every case; otherwise only the named ones)
"""
import dataclasses
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

from hermeshd_gb300 import config, ic  # noqa: E402


def cases():
    """name -> (Config, initial state, steps)."""
    c = {}
    cfg = config.sod_1d(nx=32)
    c["sod_32_hllc_rk2_nb4"] = (cfg, ic.sod(cfg), 20)
    cfg = config.sod_1d(nx=32, ihllc=2)
    c["sod_32_roe_rk2_nb4"] = (cfg, ic.sod(cfg), 20)
    cfg = config.isentropic_vortex_2d(n=8)
    c["vortex_8_rk3_nb10"] = (cfg, ic.isentropic_vortex(cfg), 10)
    cfg = config.taylor_green_3d(n=4, precision="fp64")
    c["tgv_4_ivis1_rk3_nb4"] = (cfg, ic.taylor_green(cfg, perturb=1e-3, seed=1), 10)
    cfg = config.Config(nx=4, ny=3, nz=2, nbasis=8, iquad=2, ivis=1, coll=2.0, colvis=0.5,
                        xlobc="wall", xhibc="noslip", zlobc="outflow", zhibc="wall")
    c["walls_nb8_ivis1_rk2"] = (cfg, ic.random_smooth(cfg, seed=5, amp=0.05, stress_amp=0.01), 10)
    cfg = config.Config(nx=4, ny=4, nz=3, nbasis=4, iquad=2, ivis=2, coll=1.5, colvis=1.0)
    c["tenmoment_ivis2_nb4_rk2"] = (cfg, ic.ten_moment_stress(cfg, ic.random_smooth(cfg, seed=3, amp=0.05),
                                                               p=1.0, amp=0.01), 10)
    cfg = config.Config(nx=4, ny=4, nz=3, nbasis=4, iquad=2, ivis=3, coll=2.0, iorder=2)
    c["grad_ivis3_nb4_rk2"] = (cfg, ic.ten_moment_stress(cfg, ic.random_smooth(cfg, seed=9, amp=0.05),
                                                          p=1.0, amp=0.01), 10)
    cfg = config.fh_box(4, precision="fp64", seed=42)
    c["fh_noise_4_roe_rk2_nb4"] = (cfg, ic.equilibrium(cfg), 10)
    cfg = config.poiseuille_2d(nx=8, ny=16)
    c["channel_8x16_bodyforce_rk2"] = (cfg, ic.channel(cfg, amplitude=1e-3, seed=0), 20)
    return c


def config_json(cfg):
    return json.dumps(dataclasses.asdict(cfg), sort_keys=True)


def main(names=()):
    import oracle as O
    for name, (cfg, Q0, steps) in cases().items():
        if names and name not in names:
            continue
        o = O.Oracle(cfg)
        Q0 = np.asfortranarray(Q0)
        rhs = o.rhs(Q0.copy(order="F"), limit=True)
        Q = Q0.copy(order="F")
        t, dt = o.advance(Q, steps)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, Q0=Q0, rhs=rhs, Q=Q, t=t, dt=dt, steps=steps, config=config_json(cfg))
        print(f"{name}: {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))

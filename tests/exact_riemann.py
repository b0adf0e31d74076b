"""Exact solution of the 1-D Riemann problem for an ideal gas (Toro,
"Riemann Solvers and Numerical Methods for Fluid Dynamics", ch. 4):
Newton iteration for the star pressure, then sampling.  Used to pin the
oracle and the CUDA path on the Sod shock tube."""
import math

import numpy as np


def _fK(p, rhoK, pK, g):
    cK = math.sqrt(g * pK / rhoK)
    if p > pK:  # shock
        A = 2.0 / ((g + 1) * rhoK)
        B = (g - 1) / (g + 1) * pK
        f = (p - pK) * math.sqrt(A / (p + B))
        df = math.sqrt(A / (B + p)) * (1 - (p - pK) / (2 * (B + p)))
    else:  # rarefaction
        f = 2 * cK / (g - 1) * ((p / pK) ** ((g - 1) / (2 * g)) - 1)
        df = 1.0 / (rhoK * cK) * (p / pK) ** (-(g + 1) / (2 * g))
    return f, df


def star_state(rl, ul, pl, rr, ur, pr, g):
    p = 0.5 * (pl + pr)
    for _ in range(100):
        fl, dfl = _fK(p, rl, pl, g)
        fr, dfr = _fK(p, rr, pr, g)
        dp = (fl + fr + ur - ul) / (dfl + dfr)
        p = max(p - dp, 1e-12)
        if abs(dp) < 1e-14 * p:
            break
    fl, _ = _fK(p, rl, pl, g)
    fr, _ = _fK(p, rr, pr, g)
    u = 0.5 * (ul + ur) + 0.5 * (fr - fl)
    return p, u


def sample(x, t, x0, rl, ul, pl, rr, ur, pr, g):
    """Density, velocity, pressure at positions x (array) and time t."""
    ps, us = star_state(rl, ul, pl, rr, ur, pr, g)
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    out = np.zeros((3, len(x)))
    for n, xx in enumerate(x):
        s = (xx - x0) / t
        if s <= us:
            if ps > pl:
                rsl = rl * ((ps / pl + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pl + 1))
                SL = ul - cl * math.sqrt((g + 1) / (2 * g) * ps / pl + (g - 1) / (2 * g))
                out[:, n] = (rl, ul, pl) if s <= SL else (rsl, us, ps)
            else:
                csl = cl * (ps / pl) ** ((g - 1) / (2 * g))
                SHL, STL = ul - cl, us - csl
                if s <= SHL:
                    out[:, n] = (rl, ul, pl)
                elif s > STL:
                    out[:, n] = (rl * (ps / pl) ** (1 / g), us, ps)
                else:
                    c = 2 / (g + 1) * (cl + (g - 1) / 2 * (ul - s))
                    r = rl * (2 / (g + 1) + (g - 1) / ((g + 1) * cl) * (ul - s)) ** (2 / (g - 1))
                    out[:, n] = (r, 2 / (g + 1) * (cl + (g - 1) / 2 * ul + s), pl * (c / cl) ** (2 * g / (g - 1)))
        else:
            if ps > pr:
                rsr = rr * ((ps / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pr + 1))
                SR = ur + cr * math.sqrt((g + 1) / (2 * g) * ps / pr + (g - 1) / (2 * g))
                out[:, n] = (rr, ur, pr) if s >= SR else (rsr, us, ps)
            else:
                csr = cr * (ps / pr) ** ((g - 1) / (2 * g))
                SHR, STR = ur + cr, us + csr
                if s >= SHR:
                    out[:, n] = (rr, ur, pr)
                elif s <= STR:
                    out[:, n] = (rr * (ps / pr) ** (1 / g), us, ps)
                else:
                    c = 2 / (g + 1) * (cr - (g - 1) / 2 * (ur - s))
                    r = rr * (2 / (g + 1) - (g - 1) / ((g + 1) * cr) * (ur - s)) ** (2 / (g - 1))
                    out[:, n] = (r, 2 / (g + 1) * (-cr + (g - 1) / 2 * ur + s), pr * (c / cr) ** (2 * g / (g - 1)))
    return out

"""Run-time configuration of one DG problem.

The reference fixes every parameter at compile time in ``src/input.f90`` and
``src/params.f90`` (one binary per problem; the per-problem snapshots live in
``tests/*/input_*.f90``).  :class:`Config` carries the same parameters at run
time.  Field names follow the reference's Fortran names (``iquad``,
``nbasis``, ``ivis``, ``ieos``, ``ihllc``, ``aindex``, ``rh_floor``,
``T_floor``, ``coll``, ``colvis``, ``cflm``, ``xlobc`` ...).
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass, field
from typing import Optional, Tuple

NQ = 11                      # params.f90:47
VARS = ("rh", "mx", "my", "mz", "en", "pxx", "pyy", "pzz", "pxy", "pxz", "pyz")  # params.f90:42-46
BC_CODES = {"periodic": 0, "outflow": 1, "wall": 2, "noslip": 3, "inflow": 4}
SUPPORTED_BASES = ((4, 2), (8, 2), (10, 3))          # (nbasis, iquad) with a CUDA instantiation
ORACLE_BASES = ((4, 2), (8, 2), (10, 3), (27, 3))    # the oracle also runs (27, 3)


def bc_code(name: str) -> int:
    """Map a reference BC name to its code.  boundary.f90:789-880 maps any
    unknown name to the periodic routine; so does this."""
    return BC_CODES.get(name, 0)


def default_cflm(iquad: int) -> float:
    """initialize.f90:104-122 set_cflm."""
    return {2: 0.14, 3: 0.08, 4: 0.05}.get(iquad, 0.14)


@dataclass(frozen=True)
class Units:
    """Dimensional units of params.f90:80-105 (the src/ variant).

    ``T_floor``, ``P_base`` and ``P_1`` in code units follow from the
    temperature floor ``TK`` (Kelvin) and the molecular mass ``mu`` (AMU).
    """
    TK: float = 94.4
    mu: float = 39.948
    n0: float = 2.5e25
    amu: float = 1.67e-27
    eV_per_K: float = 8.61728e-5
    J_per_eV: float = 1.6e-19
    P_atm: float = 1.01e5

    @property
    def p0(self) -> float:
        return self.mu * self.amu * self.n0          # v0 = L0/t0 = 1

    @property
    def te0(self) -> float:
        return self.p0 / self.n0 / self.J_per_eV

    @property
    def T_floor(self) -> float:
        return self.TK * self.eV_per_K / self.te0

    @property
    def P_base(self) -> float:
        return self.P_atm / self.p0

    @property
    def P_1(self) -> float:
        return 2.15e9 / 7.2 / self.p0


def units_isentropic_vortex() -> Units:
    """tests/2D_isentropic_vortex/params_isentr.f90:72-94 (TK = 1 K, mu = 18,
    SI constants k_B/J_per_eV, M_u and n_ig = 2.504e25)."""
    k_B, J_per_eV = 1.380651e-23, 1.602176e-19
    return Units(TK=1.0, mu=18.0, n0=2.504e25, amu=1.660539e-27, eV_per_K=k_B / J_per_eV,
                 J_per_eV=J_per_eV, P_atm=1.013e5)


@dataclass
class Config:
    # grid (input.f90 nx, ny, nz with one MPI domain per dimension)
    nx: int = 16
    ny: int = 16
    nz: int = 1
    lx: float = 1.0
    ly: float = 1.0
    lz: float = 1.0
    # discretisation (input.f90 iquad, nbasis; the pair picks ibitri)
    nbasis: int = 4
    iquad: int = 2
    iorder: int = 2                  # 2 'heun', 3 'shu-osher' (integrator.f90:39-55)
    # physics switches
    ivis: int = 0                    # 0 explicit, 1 semi-implicit stress, 2 10-moment, 3 Grad closure (E_ij)
    ieos: int = 1                    # 1 ideal gas, 2 Murnaghan-Tait
    ihllc: int = 1                   # 0 central/LLF, 1 HLLC, 2 Roe (the monolithic code's iroe; ideal-gas
                                     # Roe average: with ieos 2 use 0 or 1)
    aindex: float = 5.0 / 3.0        # gamma
    rh_floor: float = 5.0e-6         # params.f90:93
    T_floor: float = field(default_factory=lambda: Units().T_floor)
    rh_mult: float = 1.01            # params.f90:105
    P_1: float = field(default_factory=lambda: Units().P_1)
    P_base: float = field(default_factory=lambda: Units().P_base)
    coll: float = 0.0
    colvis: float = 0.0
    cflm: float = 0.0                # <= 0: initialize.f90 default for iquad
    # boundaries (input.f90 xlobc ... zhibc)
    xlobc: str = "periodic"
    xhibc: str = "periodic"
    ylobc: str = "periodic"
    yhibc: str = "periodic"
    zlobc: str = "periodic"
    zhibc: str = "periodic"
    # fluctuating hydrodynamics (input.f90 llns; random.f90)
    llns: bool = False
    eta_sd: float = 0.0              # stress amplitude per unit normal, already scaled by 1/sqrt(dV dt)
    zeta_sd: float = 0.0
    seed: int = 0
    # body force in x (new: the reference drives its channel by inflow)
    body_force: float = 0.0
    # parabolic x-low inflow (xlobc = "inflow"; boundary.f90:568-612): peak
    # velocity, density and pressure (<= 0: rho * T_floor, as poiseuille_flow)
    inflow_u: float = 0.3
    inflow_rho: float = 1.0
    inflow_p: float = 0.0
    # precision of the bulk arithmetic: "fp64" or "fp32"
    precision: str = "fp64"
    # simulation end time and output cadence (input.f90 tf, ntout)
    tf: float = 1.0
    ntout: int = 200

    # ---- derived -------------------------------------------------------
    @property
    def ncells(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def shape_f(self) -> Tuple[int, int, int, int, int]:
        """Fortran shape (nx, ny, nz, nQ, nbasis) of one field array."""
        return (self.nx, self.ny, self.nz, NQ, self.nbasis)

    @property
    def shape_c(self) -> Tuple[int, int, int, int, int]:
        """The same memory seen C-contiguous: (nbasis, nQ, nz, ny, nx)."""
        return (self.nbasis, NQ, self.nz, self.ny, self.nx)

    @property
    def dof(self) -> int:
        return self.ncells * NQ * self.nbasis

    @property
    def stages(self) -> int:
        return 3 if self.iorder == 3 else 2

    @property
    def cflm_eff(self) -> float:
        return self.cflm if self.cflm > 0 else default_cflm(self.iquad)

    @property
    def inflow_pressure(self) -> float:
        return self.inflow_p if self.inflow_p > 0 else self.inflow_rho * self.T_floor

    @property
    def bc(self) -> Tuple[int, ...]:
        return tuple(bc_code(s) for s in (self.xlobc, self.xhibc, self.ylobc, self.yhibc, self.zlobc, self.zhibc))

    def replace(self, **kw) -> "Config":
        return dataclasses.replace(self, **kw)

    def validate(self, oracle: bool = False) -> None:
        allowed = ORACLE_BASES if oracle else SUPPORTED_BASES
        if (self.nbasis, self.iquad) not in allowed:
            raise ValueError(f"(nbasis, iquad) = ({self.nbasis}, {self.iquad}) not in {allowed}")
        if min(self.nx, self.ny, self.nz) < 1:
            raise ValueError("grid dimensions must be >= 1")
        if self.ivis not in (0, 1, 2, 3) or self.ieos not in (1, 2) or self.iorder not in (2, 3):
            raise ValueError("ivis in {0,1,2,3}, ieos in {1,2}, iorder in {2,3}")
        if int(self.ihllc) not in (0, 1, 2):
            raise ValueError("ihllc in {0 central/LLF, 1 HLLC, 2 Roe}")
        if self.precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        if "inflow" in (self.xhibc, self.ylobc, self.yhibc, self.zlobc, self.zhibc):
            raise ValueError("the inflow boundary is defined for the x-low face only")


# ---------------------------------------------------------------------------
# Problem presets: the five benchmark configurations
# ---------------------------------------------------------------------------

def sod_1d(nx: int = 256, **kw) -> Config:
    """1-D Sod shock tube, 5-moment, linear basis, HLLC, SSP-RK2, CFL 0.3.

    Follows tests/1D_sod_shock_tube/input_sod.f90 (lx = 1, ly = lx/12,
    lz = lx/120, gamma 5/3, TK 300, mu 18, wall x-ends, periodic y/z) with
    pressure measured in units of the reference's P_base: the reference's IC
    sets p = P_base*{1, 0.1} (initialcon.f90:196-199); here p = {1, 0.1} and
    the temperature floor is divided by P_base, which is the same problem
    with velocity and time rescaled by sqrt(P_base)."""
    u = Units(TK=300.0, mu=18.0)
    c = Config(nx=nx, ny=1, nz=1, lx=1.0, ly=1.0 / 12.0, lz=1.0 / 120.0, nbasis=4, iquad=2, iorder=2,
               ivis=0, ieos=1, ihllc=1, aindex=5.0 / 3.0, T_floor=u.T_floor / u.P_base,
               P_1=u.P_1 / u.P_base, P_base=1.0, cflm=0.3, xlobc="wall", xhibc="wall", tf=0.2)
    return c.replace(**kw)


def isentropic_vortex_2d(n: int = 128, precision: str = "fp64", **kw) -> Config:
    """2-D isentropic vortex (initialcon.f90:128-183, version 1: mean flow
    (1,1), Rgsqi 0.5, beta 5), periodic [-5,5]^2, quadratic basis (nb 10,
    iquad 3), HLLC, SSP-RK3, one period t = 10.  gamma 7/5 and the floors of
    tests/2D_isentropic_vortex/{input,params}_isentr.f90."""
    u = units_isentropic_vortex()
    c = Config(nx=n, ny=n, nz=1, lx=10.0, ly=10.0, lz=10.0 / 120.0, nbasis=10, iquad=3, iorder=3,
               ivis=0, ieos=1, ihllc=1, aindex=7.0 / 5.0, T_floor=u.T_floor, P_1=u.P_1, P_base=u.P_base,
               tf=10.0, precision=precision)
    return c.replace(**kw)


def taylor_green_3d(n: int = 64, precision: str = "fp32", mach: float = 0.1, reynolds: float = 400.0, **kw) -> Config:
    """3-D Taylor-Green vortex, 10-moment relaxation (ivis 1), linear basis,
    periodic [0,2pi]^3, Mach 0.1 (V0 = 1, c = 10), Re 400 with L = 1.
    p = rho c^2 / gamma; mu = rho V0 L / Re; coll = p/mu; colvis = p (the
    pattern of initialcon.f90:89-90).  No reference IC exists for this case."""
    gamma = 5.0 / 3.0
    cs = 1.0 / mach
    p = cs * cs / gamma
    mu = 1.0 / reynolds
    L = 2.0 * math.pi
    c = Config(nx=n, ny=n, nz=n, lx=L, ly=L, lz=L, nbasis=4, iquad=2, iorder=3, ivis=1, ieos=1, ihllc=1,
               aindex=gamma, coll=p / mu, colvis=p, precision=precision)
    return c.replace(**kw)


def fh_box(n: int, eta: float = 1.0, kT_over_rho_dV: float = 1.0e-3, seed: int = 0, dt_noise: float = 0.1,
           precision: str = "fp32", ihllc: int = 2, **kw) -> Config:
    """One realisation of the fluctuating-hydro ensemble: 10-moment (ivis 1)
    with stochastic stress, equilibrium rho = 1, T = 1 (p = 1), v = 0, nb 4.
    kT/(rho dV) = 1e-3 fixes the cell volume dV = 1000 (dx = 10).  The shear
    viscosity eta is not given by the benchmark; eta = 1 is chosen.
    Amplitude per unit normal: sqrt(2 eta kT / (dV dt_noise)).

    Riemann solver: Roe (ihllc = 2).  The reference's HLLC receives the
    stress-augmented point flux, whose star fluxes differ by P_dd,L - P_dd,R
    on the two sides of S_M = 0 (flux.f90:87-89,623-643); an equilibrium
    fluctuating state has S_M ~ 0 at every face, so with HLLC the branch is
    picked by rounding and FP32 and FP64 runs part at ~1e-4 in ensemble
    means, against ~1e-7 with the Roe solver, which is continuous there."""
    gamma = 5.0 / 3.0
    dV = 1.0 / kT_over_rho_dV
    dx = dV ** (1.0 / 3.0)
    L = n * dx
    p = 1.0
    eta_sd = math.sqrt(2.0 * eta * 1.0 / (dV * dt_noise))
    c = Config(nx=n, ny=n, nz=n, lx=L, ly=L, lz=L, nbasis=4, iquad=2, iorder=2, ivis=1, ieos=1, ihllc=ihllc,
               aindex=gamma, coll=p / eta, colvis=p, llns=True, eta_sd=eta_sd, zeta_sd=0.0, seed=seed,
               precision=precision)
    return c.replace(**kw)


def poiseuille_2d(nx: int = 64, ny: int = 128, viscosity: float = 0.05, body_force: float = 1.0e-3,
                  ihllc: int = 2, **kw) -> Config:
    """2-D channel: periodic x, no-slip walls in y (boundary.f90:100-122),
    10-moment ivis 1 where viscosity enters through coll = p/mu (colvis = p),
    driven by a uniform body force in x.  rho = 1, p = 1, ly = 1.

    The cells are square (lx = ly*nx/ny): the reference's time step uses the
    x spacing only (hermeshd.f90:174), so cells thinner in y than in x run
    above the stable CFL number in y (with lx = 2, a 16x32 grid's velocities
    grow from 1e-3 to 0.06-0.25 within 40 steps).  Roe flux
    (ihllc = 2) by default: with the stress-augmented point flux HLLC is
    discontinuous at S_M = 0 (flux.f90:623-643), which at rest is everywhere
    in the channel, and it amplifies the perturbation (1e-3 to 2.5e-2 in 240
    steps on a 16x32 grid) where Roe and the central flux damp it."""
    p = 1.0
    ly = 1.0
    c = Config(nx=nx, ny=ny, nz=1, lx=ly * nx / ny, ly=ly, lz=1.0 / 120.0, nbasis=4, iquad=2, iorder=2, ivis=1,
               ieos=1, ihllc=ihllc, aindex=5.0 / 3.0, coll=p / viscosity, colvis=p, ylobc="noslip",
               yhibc="noslip", body_force=body_force)
    return c.replace(**kw)

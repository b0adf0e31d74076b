/*
 * hermes_oracle.h -- CPU FP64 restatement of the HERMESHD DG step (TEST
 * INFRASTRUCTURE ONLY).
 *
 * This library is the checker for the CUDA path and the timed CPU baseline.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may
 * load it; the product library (hermeshd_gb300) never links or calls it.
 *
 * Every routine follows the reference Fortran loop by loop (file:line given
 * in hermes_oracle.c), with REAL4 promoted to double.  Arrays use the
 * reference's Fortran layout Q(nx,ny,nz,nQ,nbasis): x fastest, basis slowest.
 *
 * Parity pinning: the reference ships no golden vectors and cannot be built
 * here (no Fortran compiler, MPI or MKL).  The oracle is pinned by the
 * reference's own known-answer self-test (basis orthonormality,
 * basis_funcs.f90:634-992), by analytic solutions (exact Sod Riemann
 * solution, exactly advected isentropic vortex) and by conservation; see
 * tests/test_oracle_kat.py.
 */
#ifndef HERMES_ORACLE_H
#define HERMES_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_NQ = 11, ORC_NBASTOT = 30 };

/* boundary condition codes, boundary.f90:789-880 (unknown names -> periodic) */
enum { ORC_BC_PERIODIC = 0, ORC_BC_OUTFLOW = 1, ORC_BC_WALL = 2, ORC_BC_NOSLIP = 3, ORC_BC_INFLOW = 4 };

typedef struct orc_params {
    int nx, ny, nz;          /* cells (input.f90 nx,ny,nz with mpi_n* = 1) */
    int nbasis, iquad;       /* (4,2) (8,2) (10,3) (27,3) */
    int ivis;                /* 0 explicit, 1 semi-implicit stress, 2 10-moment, 3 Grad closure */
    int ieos;                /* 1 ideal gas, 2 Murnaghan-Tait */
    int ihllc;               /* 0 central/LLF, 1 HLLC (flux.f90:264-271), 2 Roe (SEAN monolith) */
    int iorder;              /* 2 Heun (RK2), 3 Shu-Osher (RK3) */
    int bc[6];               /* xlo, xhi, ylo, yhi, zlo, zhi */
    double lx, ly, lz;       /* domain lengths, domain centred at 0 */
    double aindex;           /* gamma */
    double rh_floor, T_floor;
    double coll, colvis;     /* relaxation rate and coll*viscosity */
    double cflm;             /* <= 0 selects the reference default for iquad */
    double P_1, P_base;      /* Tait EOS constants (ieos 2) */
    double rh_mult;          /* density multiplier in get_min_dt */
    int llns;                /* 1: stochastic stress in the point fluxes */
    int pad_;
    double eta_sd, zeta_sd;  /* stochastic stress amplitudes (already scaled) */
    unsigned long long seed; /* Philox key for the stochastic stress */
    double body_force;       /* uniform x body force (no reference counterpart) */
    double inflow_u, inflow_rho, inflow_p;   /* x-low inflow profile (boundary.f90:568-612) */
} orc_params;

typedef struct orc_ctx orc_ctx;

orc_ctx *orc_create(const orc_params *p);
void orc_destroy(orc_ctx *c);

/* sizes: number of doubles in one Q array */
long orc_qsize(const orc_ctx *c);
double orc_cflm(const orc_ctx *c);

/* tables (for tests); rows x nbastot, row-major [row][basis] */
int orc_get_table(const orc_ctx *c, const char *name, double *out, int maxn);
int orc_get_kindex(const orc_ctx *c, int *out30);  /* kx.. indices, 1-based */

/* the pieces of one forward-Euler stage (integrator.f90:93-122) */
void orc_limiter(orc_ctx *c, double *Q);
void orc_prep_and_rhs(orc_ctx *c, double *Q, double *rhs_out);   /* limiter+exchange+bc+glflux+source; rhs = glflux - source */
void orc_rhs_nolimit(orc_ctx *c, const double *Q, double *rhs_out); /* exchange+bc+glflux+source only */
void orc_euler_step(orc_ctx *c, double *Qin, double *Qout, double dt);
double orc_get_min_dt(orc_ctx *c, const double *Q);
/* hermeshd.f90:53-62: dt = get_min_dt(Q); update(Q,Q1,Q2,dt); t += dt */
void orc_step(orc_ctx *c, double *Q, double *Q1, double *Q2, double *t, double *dt);
/* nsteps of step(); returns number of steps taken */
int orc_advance(orc_ctx *c, double *Q, double *Q1, double *Q2, double *t, double *dt, int nsteps);
/* run with a fixed dt (no CFL): nsteps RK steps */
void orc_advance_fixed_dt(orc_ctx *c, double *Q, double *Q1, double *Q2, double dt, int nsteps);
/* counter for the stochastic stress; the (step, stage) part of the Philox counter */
void orc_set_noise_counter(orc_ctx *c, unsigned long long step);

/* nine Philox normals and the stochastic stress {xx,yy,zz,xy,xz,yz} of one
 * quadrature point of one flux call (for statistical tests) */
void orc_noise_sample(unsigned long long seed, unsigned long long step, unsigned stage, unsigned kind,
                      unsigned long long site, unsigned pt, double eta, double zeta, double G6[6], double S6[6]);
/* one Philox-4x32-10 block (known-answer tests) */
void orc_philox4x32_10(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]);

/* per-phase wall time accumulators (seconds): limiter, faces, volume, surface, source, update */
void orc_get_timers(const orc_ctx *c, double *out6);
void orc_reset_timers(orc_ctx *c);
int orc_num_threads(void);
void orc_set_num_threads(int n);

/* the reference's basis self-test (basis_funcs.f90:634-992): returns the
 * maximum absolute deviation of the cell and face scalar products from the
 * expected identity pattern */
double orc_test_basis(const orc_ctx *c, double *cell_dev, double *face_dev);

#ifdef __cplusplus
}
#endif
#endif

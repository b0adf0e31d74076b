/*
 * hermes_gb300.h -- C ABI of the GB300 DG right-hand side and SSP-RK time
 * step of HERMESHD (5- and 10-moment systems).
 *
 * This is the drop-in boundary for the reference's step path.  The
 * reference exposes that path to Python through an f2py/f90wrap extension
 * (src/hermeshd.py:5-120, wrapping src/hermeshd.f90:26-199); the Python
 * package hermeshd_gb300 binds the functions below with ctypes and keeps the
 * reference's call surface on top of them.
 *
 * Conventions
 *  - Field arrays use the reference layout Q(nx,ny,nz,nQ,nbasis) in Fortran
 *    order (x fastest, basis slowest), nQ = 11 variables rh, mx, my, mz, en,
 *    pxx, pyy, pzz, pxy, pxz, pyz (params.f90:42-47).  Element type is double
 *    when cfg->precision == 64 and float when it is 32.
 *  - Pointers named q* are device pointers unless the function name ends in
 *    _host.  Device work is ordered after, and before, the caller's stream.
 *  - Every function returns a hermes_status code; the reference returns none
 *    and calls exit(-1) on a NaN (integrator.f90:234-250).  The message of
 *    the last failure is hermes_last_error(ctx).
 *  - No entry point exits, traps or aborts the process.
 */
#ifndef HERMES_GB300_H
#define HERMES_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HERMES_ABI_VERSION 8

typedef enum hermes_status {
    HERMES_OK = 0,
    HERMES_ERR_CONFIG = 1,     /* unsupported or inconsistent configuration */
    HERMES_ERR_SHAPE = 2,      /* array size does not match the configuration */
    HERMES_ERR_DTYPE = 3,      /* element type does not match cfg->precision */
    HERMES_ERR_NONFINITE = 4,  /* a NaN cell average appeared (integrator.f90:234-250) */
    HERMES_ERR_TIMEOUT = 5,    /* a bounded device wait ran out */
    HERMES_ERR_CUDA = 6,       /* a CUDA runtime call failed */
    HERMES_ERR_ALLOC = 7,      /* device or host allocation failed */
    HERMES_ERR_ARG = 8         /* null pointer or invalid argument */
} hermes_status;

/* boundary condition codes: boundary.f90:789-880 ('periodic', 'outflow',
 * 'wall', 'noslip'; any other name selects periodic there, and here), and
 * the parabolic inflow of boundary_custom (boundary.f90:568-612 x_bc_inflow /
 * set_xlobc_inflow), which the reference defines but does not select: x-low
 * face only, one grid. */
enum { HERMES_BC_PERIODIC = 0, HERMES_BC_OUTFLOW = 1, HERMES_BC_WALL = 2, HERMES_BC_NOSLIP = 3, HERMES_BC_INFLOW = 4 };

/* The run-time form of the reference's compile-time configuration
 * (src/input.f90, src/params.f90, tests/<problem>/input_*.f90). */
typedef struct hermes_config {
    int32_t nx, ny, nz;        /* cells; input.f90 nx, ny, nz with one MPI domain */
    int32_t nbasis, iquad;     /* (4,2), (8,2) or (10,3): input.f90 nbasis, iquad */
    int32_t iorder;            /* 2 'heun' or 3 'shu-osher': integrator.f90:39-55 */
    int32_t ivis;              /* 0, 1, 2: input.f90 ivis; 3: Grad closure (E_ij form with an implicit
                                  source step after each RK2 stage) of src/ces/10_moment/
                                  dg_3D_hydro_bitri_ten_moment.f90 (its ivis 0) */
    int32_t ieos;              /* 1 ideal gas, 2 Murnaghan-Tait */
    int32_t ihllc;             /* Riemann solver for rh..en: 0 central/LLF only, 1 HLLC (flux.f90:264-271),
                                  2 Roe (src/ces/10_moment/dg_3D_hydro_lqc_SEAN.f90:1614-1789; its Roe
                                  average is the ideal-gas one, so with ieos 2 it does not carry the
                                  Tait sound speed: use 0 or 1 there) */
    int32_t bc[6];             /* xlo, xhi, ylo, yhi, zlo, zhi: HERMES_BC_* */
    int32_t precision;         /* 64 (FP64) or 32 (FP32 bulk, FP64 CFL and limiter fixes) */
    int32_t llns;              /* nonzero: stochastic stress (random.f90:106-145) */
    double lx, ly, lz;         /* domain lengths; the domain is centred at 0 */
    double aindex;             /* gamma */
    double rh_floor, T_floor;  /* params.f90:93-95 */
    double rh_mult;            /* params.f90:105 */
    double coll, colvis;       /* relaxation rate, coll*viscosity (params.f90:115) */
    double cflm;               /* <= 0: initialize.f90:104-122 default for iquad */
    double P_1, P_base;        /* Tait EOS constants (params.f90:104) */
    double eta_sd, zeta_sd;    /* stochastic stress amplitudes per unit normal */
    uint64_t seed;             /* Philox key of the stochastic stress */
    double body_force;         /* uniform x body force (no reference counterpart) */
    double inflow_u;           /* HERMES_BC_INFLOW: peak velocity ux_amb of the profile 4u y(ly-y)/ly^2 */
    double inflow_rho;         /* HERMES_BC_INFLOW: density */
    double inflow_p;           /* HERMES_BC_INFLOW: pressure */
} hermes_config;

typedef struct hermes_ctx hermes_ctx;

/* ABI version of the loaded library (HERMES_ABI_VERSION). */
int hermes_abi_version(void);

/* sizeof(hermes_config) as compiled into the library (binding check). */
int hermes_config_size(void);

/* Number of elements of one field array for cfg, and the device scratch the
 * context allocates (face-flux buffers).  No device work. */
int hermes_sizes(const hermes_config *cfg, size_t *q_elems, size_t *scratch_bytes);

/* Create a context: the GB300 replacement of setup()'s discretisation part
 * (hermeshd.f90:67-114 -> initialize.f90:24-61 initializer: basis tables,
 * cbasis, cflm, grid spacing).  Initial conditions stay with the caller, as
 * in the f90wrap interface where Q_io is caller-owned.  stream: the
 * caller's cudaStream_t (NULL = the legacy default stream).  The context
 * runs its kernels on a private stream that waits for the caller's stream at
 * the start of every call and that the caller's stream waits for at the end,
 * so calls are stream-ordered with the caller's own work. */
int hermes_create(const hermes_config *cfg, void *stream, hermes_ctx **out);

/* An ensemble of nbox independent grids sharing cfg's physics, advanced
 * together: dims[3*i..3*i+2] = (nx, ny, nz) of box i, seeds[i] its Philox
 * key (NULL: cfg->seed + i), lengths[3*i..] its domain lengths (NULL: cfg's).
 * Field arrays hold the boxes back to back, box i starting at element
 * offsets[i] (hermes_box_offsets).  No reference counterpart (batching). */
int hermes_ensemble_create(const hermes_config *cfg, int nbox, const int32_t *dims, const double *lengths,
                           const uint64_t *seeds, void *stream, hermes_ctx **out);
int hermes_box_offsets(hermes_ctx *ctx, int64_t *offsets /* nbox+1 */);

int hermes_destroy(hermes_ctx *ctx);

/* Message of the last failure on this context (static storage of the ctx). */
const char *hermes_last_error(hermes_ctx *ctx);

/* The context's private CUDA stream (cudaStream_t) its kernels run on. */
void *hermes_stream(hermes_ctx *ctx);

/* get_min_dt (hermeshd.f90:145-199): CFL time step from the cell averages
 * of q, in FP64, including the reference's use of the last cell's sound
 * speed and of dxi only.  Synchronises; dt_out is a host pointer. */
int hermes_get_min_dt(hermes_ctx *ctx, const void *q, double *dt_out);

/* limiter (flux.f90:1077-1164), in place on q. */
int hermes_limiter(hermes_ctx *ctx, void *q);

/* calc_rhs (integrator.f90:116-122 -> glflux flux.f90:932-1022 and
 * source_calc sources.f90:12-84) after prep_advance's limiter when
 * apply_limiter is nonzero (integrator.f90:106-113): rhs = glflux_r -
 * source_r, in the layout of q.  q is limited in place, as in the reference. */
int hermes_rhs(hermes_ctx *ctx, void *q, void *rhs, int apply_limiter);

/* euler_step (integrator.f90:93-102): q_out = advance_time_level(lim(q_in)). */
int hermes_euler_stage(hermes_ctx *ctx, void *q_in, void *q_out, double dt);

/* step (hermeshd.f90:53-62, f90wrap_step in hermeshd.py:31-47): dt =
 * get_min_dt(q); update(q, q1, q2, dt) with RK2 or RK3 (integrator.f90:62-86);
 * t += dt.  t and dt are host scalars, read and written as in the reference.
 * q1 and q2 are caller-provided scratch, as there; q2 is left unwritten.
 * Synchronises (to return dt and t). */
int hermes_step(hermes_ctx *ctx, void *q, void *q1, void *q2, double *t, double *dt);

/* nsteps of step() from one CUDA graph, one synchronisation at the end
 * (the loop of hermeshd.f90:38-41 without output). */
int hermes_advance(hermes_ctx *ctx, void *q, void *q1, void *q2, int nsteps, double *t, double *dt);

/* The same with host buffers: q_host (nsteps of step() on a device copy,
 * then copied back, with one synchronisation; a state with a NaN cell
 * average is copied back as well and HERMES_ERR_NONFINITE returned).  When
 * q_host is pinned memory mapped into the device's address space
 * (cudaHostAlloc, cudaHostRegister with cudaHostRegisterMapped), the last
 * stage stores the new state into it directly, the copy back overlapping
 * that kernel; other host memory is copied back after the steps.  The
 * reference's interface takes host arrays. */
int hermes_advance_host(hermes_ctx *ctx, void *q_host, int nsteps, double *t, double *dt);

/* nsteps of step() enqueued on the context's stream from the CUDA graph,
 * without synchronising; t and dt stay on the device (hermes_box_times). */
int hermes_enqueue_steps(hermes_ctx *ctx, void *q, void *q1, int nsteps);

/* Text checkpoints of writeQ / readQ (initialize.f90:474-565), host memory
 * only (no context, no GPU).  q: FP64 Q(nx,ny,nz,nQ,nbasis), Fortran order.
 * Records: one per (basis, variable, k, j) with the nx values of the row,
 * then "t dt nout mpi_nx mpi_ny mpi_nz".  The writer prints %.16E (exact FP64
 * round trip); the reader accepts Fortran list-directed input (blank or comma
 * separators, continuation lines, r*c repeats, null values, D exponents, a
 * slash ending a list), so files the reference wrote read back.  mpi_dims: 3
 * values (NULL = 1 1 1 on write).  err (errlen bytes, may be NULL) receives a
 * message on failure; a short or malformed file returns HERMES_ERR_SHAPE. */
int hermes_checkpoint_write(const char *path, const double *q, int32_t nx, int32_t ny, int32_t nz, int32_t nbasis,
                            double t, double dt, int32_t nout, const int32_t *mpi_dims, char *err, size_t errlen);
int hermes_checkpoint_read(const char *path, double *q, int32_t nx, int32_t ny, int32_t nz, int32_t nbasis,
                           double *t, double *dt, int32_t *nout, int32_t *mpi_dims, char *err, size_t errlen);

/* Initial state of set_ic (initialcon.f90:20-361) built on the device for
 * every box of the context: icid 0 hydrodynamic jet (its random kick from
 * Philox-4x32-10 keyed by seed, where the reference uses Fortran's unseeded
 * random_number), 1/2 isentropic vortex versions 0/1, 3/4 Sod shock tube
 * versions 0/1, 5-7 fluid at rest (Poiseuille and cylinder problems).  Cell
 * averages only; all other coefficients are written zero. */
int hermes_init_state(hermes_ctx *ctx, void *q, int32_t icid, uint64_t seed);

/* Conservation sums in FP64 whatever the precision of q: per box, the
 * integrals of rho, m_x, m_y, m_z and E (cell averages times the cell
 * volume), 5 doubles per box into the host array sums, summed in a fixed
 * order (the same bits on every call).  No counterpart in the reference.
 * Synchronises. */
int hermes_conserved(hermes_ctx *ctx, const void *q, double *sums);

/* Derived fields of the VTK output (output.f90:14-317), on the device.  The
 * state q of a one-grid context is evaluated at nvtk^3 sub-points per cell
 * (nvtk 1..4, basis_funcs.f90:88-200) and the variables selected by mask
 * (bit v = variable v below) are written to the device array out as float32,
 * one array of nx*ny*nz*nvtk^3 values per selected variable in variable
 * order, sub-cells x fastest.  Variables: 0 density*n0, 1 log10 density*n0,
 * 2-4 velocity*v0, 5 temperature (K), 6 internal energy density, 7 total
 * energy density, 8 entropy density, 9 pressure, 10-12 diagonal stresses,
 * 13 vorticity.  (The reference never fills the internal-energy array and
 * writes the previous variable's values under that name; here it is
 * E - rho v^2/2.) */
typedef struct hermes_output_units {
    double n0, v0, t0, te0, eV_per_K;   /* params.f90:80-94 */
} hermes_output_units;
#define HERMES_DERIVED_NVARS 14
int hermes_derived(hermes_ctx *ctx, const void *q, float *out, int32_t nvtk, uint32_t mask,
                   const hermes_output_units *units);

/* Launch shape of a context, chosen by the autotuner (hermeshd_gb300/autotune.py)
 * or by hand.  No counterpart in the reference (its loops have no launch
 * shape).  Zero sizes (face_tpb, dt_tpb, steps_per_graph, update_tpb) select the
 * compiled defaults; the switches take the values given (start from
 * hermes_get_launch to change one).  Changing face_tpb or
 * dt_tpb synchronises the context's stream and drops its captured graphs. */
typedef struct hermes_launch {
    int32_t face_tpb;        /* faces per block of the face kernels: 32, 64 or 128 (default 128) */
    int32_t dt_tpb;          /* cells per block of the CFL reduction: multiple of 32 up to 256 (default 256) */
    int32_t steps_per_graph; /* whole steps per CUDA graph in hermes_advance/hermes_enqueue_steps: 1..64 (default 1) */
    int32_t noise_inline;    /* stochastic stress: 0 drawn by kernels of its own and staged in device
                                memory (default; the buffers are allocated at creation), 1 drawn inside
                                the face and cell kernels.  The same numbers either way. */
    int32_t face_traces;     /* 1: the face traces of every cell are evaluated once per stage by a
                                kernel of their own and read by the face kernels (FP64, nbasis 8/10,
                                no stochastic stress; the default there, the buffer is allocated at
                                creation); 0: the face kernels evaluate them.  Equal to rounding. */
    int32_t split_update;    /* 1: the cell update in two kernels, the volume terms (k_cell) and the
                                surface sums + update (k_update, one thread per cell and variable);
                                ivis 0/1 without the stochastic stress, and with it in FP32 and in
                                FP64 for nbasis 4; the default there (the buffer is allocated at
                                creation); 0: one kernel.
                                Bit-identical. */
    int32_t tile_stage;      /* 1: each RK stage as one fused kernel over tiles of 8x8x4 cells (faces,
                                surface and volume quadrature, update, RK combination and the next
                                stage's limiter; the stochastic stress drawn in place), the CFL
                                reduction fused with the first stage's limiter; nbasis 4, ivis 0/1
                                (a third state is allocated at creation).  Off by default: slower
                                than the separate kernels on the measured workloads; the autotuner
                                tries it.  0: the separate kernels.  Equal to rounding. */
    int32_t pdl;             /* 1: the step's kernels use programmatic dependent launch (each may
                                start launching while the one before it finishes, and waits for its
                                results before touching memory); 0 (default, measured neutral on
                                the benchmarked step): plain launches.  Bit-identical. */
    int32_t faces_merged;    /* the face kernels: 1 the three directions in one launch (the default
                                in FP64, where the directions fill each other's tails); 0 one
                                launch per direction, thread per (face, point) (nbasis 8/10 in
                                FP32, and nbasis 4 in FP32 below 2^15 cells); 2 one launch per
                                direction, thread per face looping over its points (nbasis 4 in
                                FP32 from 2^15 cells; needs the stochastic stress drawn in
                                place or absent and no trace buffer, else as 0).  Bit-identical. */
    int32_t update_tpb;      /* threads per block of the split update's k_update (one thread per cell
                                and variable): 64, 128 or 256; 0 the default (64 in FP32, 128 in
                                FP64).  Bit-identical. */
    int32_t cell_concurrent; /* 1 (default): with the split update, each stage's volume kernel runs on
                                a second stream beside the trace and face kernels (it needs neither),
                                and the update joins them, so the face kernels' small blocks fill the
                                volume kernel's tail; 0: one stream.  Bit-identical. */
} hermes_launch;
int hermes_set_launch(hermes_ctx *ctx, const hermes_launch *launch);
int hermes_get_launch(hermes_ctx *ctx, hermes_launch *launch);

/* Per-kernel device timing with CUDA events on the context's stream.  While
 * enabled, steps run without the graph and every kernel launch is bracketed
 * by an event pair.  hermes_profile_read synchronises, returns accumulated
 * milliseconds and launch counts per kernel kind and resets them.  Kinds:
 * 0 CFL reduction (with the fused stage: and the first stage's limiter), 1 limiter,
 * 2 x faces, 3 y faces, 4 z faces, 5 cell update, 6 staged stochastic stress (the
 * four noise kernels of a stage), 7 face traces, 8 fused stage. */
int hermes_profile_enable(hermes_ctx *ctx, int enable);
int hermes_profile_read(hermes_ctx *ctx, double *ms /* [9] */, int64_t *launches /* [9] */);

/* Per-box time and last time step of an ensemble (nbox entries each). */
int hermes_box_times(hermes_ctx *ctx, double *t, double *dt);
/* Set the time of every box (device) */
int hermes_set_time(hermes_ctx *ctx, double t);

/* Step counter of the stochastic-stress Philox stream (the number of
 * completed steps; stages are counted within a step). */
int hermes_set_noise_step(hermes_ctx *ctx, uint64_t step);
/* Stage index (0, 1 or 2; default 0) of the Philox counters with which
 * hermes_rhs, hermes_euler_stage and the adjoint entry points draw the
 * stochastic stress; with hermes_set_noise_step it names the draw of any
 * stage of any step (hermes_step and hermes_advance count their own stages). */
int hermes_set_noise_stage(hermes_ctx *ctx, int32_t stage);

/* Device error flags raised since the last call (HERMES_ERR_NONFINITE if a
 * NaN cell average was produced), cleared on read.  Synchronises. */
int hermes_check(hermes_ctx *ctx);

/* The right-hand side of hermes_rhs for one grid, computed without a
 * context and without allocating any device memory.  No counterpart in the
 * reference.  For callers that cannot allocate device memory when they need
 * a right-hand side: a host code whose device memory belongs to its own
 * framework or pool (for example a Fortran/MPI driver calling through its FFI
 * under a fixed memory budget), or a time loop that must not pay
 * cudaMalloc's device-wide synchronisation.
 *
 * q, rhs: device arrays of cfg's grid (q limited in place when apply_limiter);
 * stream: the cudaStream_t to run on (NULL = legacy default stream); the call
 * returns without synchronising.  The face-flux scratch lives in a static
 * device array of HERMES_NOALLOC_SCRATCH_BYTES that every GPU loading the
 * library holds until exit; a grid whose face fluxes do not fit returns
 * HERMES_ERR_SHAPE.  All calls share that array: calls that overlap on the GPU
 * race.  The first call on a device looks up the array's device address and
 * should come before any stream capture.  err (errlen bytes, may be NULL)
 * receives a message on failure.  The right-hand side is returned as
 * computed: a non-finite value in it is not reported (the reference checks
 * for NaN in the update, integrator.f90:234-250, not in the right-hand side).
 * With the stochastic stress on (cfg->llns), every call draws the same
 * realisation, the one of step 0, stage 0 (what hermes_rhs draws on a fresh
 * context). */
#define HERMES_NOALLOC_SCRATCH_BYTES (64ull << 20)
int hermes_rhs_noalloc(const hermes_config *cfg, void *q, void *rhs, int apply_limiter, void *stream, char *err,
                       size_t errlen);

/* Adjoint of the right-hand side and of one forward-Euler stage (FP64, one
 * grid, ivis 0, 1 or 2, ieos 1 or 2 but not ieos 2 with HLLC; a direction is
 * periodic at both ends or at neither).  With the stochastic stress on, the
 * realisation is held fixed: the one of the context's noise counters
 * (hermes_set_noise_step, hermes_set_noise_stage), as hermes_rhs and
 * hermes_euler_stage draw it.  No
 * counterpart in the reference, which has no derivatives; the forward map
 * they differentiate is hermes_rhs without the limiter (flux.f90:932-1022,
 * sources.f90:12-84) and the update of integrator.f90:147-224.  Branches
 * (HLLC wave selection, Roe |lambda|, the LLF maximum, floors, outflow
 * ghosts) are differentiated on their active side.  ivis 0/1 with ieos 1 use
 * hand-derived reverse sweeps; ivis 2, ieos 2 and the stochastic stress one
 * dual-number pass per column of every variable through the forward physics.
 *
 * hermes_rhs_vjp: nu = (dR/dq)^T mu for R = hermes_rhs(q) (apply_limiter 0).
 * hermes_stage_vjp: lam_in = (dE/dq_in)^T lam_out for the stage
 * E(q_in) = M (q_in - dt R(q_in)), M = faci = 1/(1 + dt coll) on the
 * stresses for ivis 1; for ivis 2 faci on the off-diagonal stresses and
 * faci (I + (coll dt / 3) J) on (pxx, pyy, pzz), J the 3x3 matrix of ones;
 * the identity elsewhere.  e_out = E(q_in) (may be NULL when dcoll is NULL);
 * dcoll, if not NULL, receives lam_out . dE/dcoll (through M for ivis 1 and
 * 2, through R for ivis 0 and 2), and the call then synchronises.  lam_in may alias lam_out.  Scratch (2x the face-flux size
 * plus one field) is allocated on the first call. */
int hermes_rhs_vjp(hermes_ctx *ctx, const void *q, const void *mu, void *nu);
/* lam_in = (dL/dq)^T lam_out for the positivity limiter L (flux.f90:1077-1164)
 * applied in place at q, the stage input before limiting: the derivative of the
 * branch the limiter takes at q (identity where it leaves the cell unchanged;
 * the arg-min face point, the clamp of theta and the floors followed as the
 * forward pass takes them).  lam_in may alias lam_out, not q. */
int hermes_limiter_vjp(hermes_ctx *ctx, const void *q, const void *lam_out, void *lam_in);
int hermes_stage_vjp(hermes_ctx *ctx, const void *q_in, const void *e_out, const void *lam_out, void *lam_in, double dt,
                     double *dcoll);

#ifdef __cplusplus
}
#endif
#endif

/*
 * hermes_oracle.c -- CPU FP64 restatement of the HERMESHD DG right-hand side
 * and SSP-RK step.  TEST INFRASTRUCTURE ONLY: the checker for the CUDA path
 * and the timed CPU baseline; nothing in the product library calls it.
 *
 * Each function names the reference routine (file:line, paths relative to the
 * HERMESHD source tree) whose loops it restates.  REAL4 is promoted to double.
 * Layout is the reference's Fortran Q(nx,ny,nz,nQ,nbasis).
 *
 * Parity pinning: the reference ships no golden vectors and cannot be
 * compiled here, so its routines are executed from their Fortran source by a
 * statement-by-statement translator (tests/golden/fortran_subset.py); the
 * tables, limiter, face fluxes, right-hand side and whole steps it produces
 * are this file's bit for bit on the cases in tests/golden/reference/
 * (tests/test_reference_vectors.py).  Also: the reference's basis self-test
 * (basis_funcs.f90:634-992), analytic solutions, conservation and a second,
 * numpy restatement of every routine.
 *
 * Build: gcc -O3 -fopenmp -ffp-contract=off -shared -fPIC (oracle/Makefile).
 * -ffp-contract=off keeps x86 and Arm results identical.
 */
#include "hermes_oracle.h"
#include "philox_ref.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NQ ORC_NQ
#define NBT ORC_NBASTOT
/* variable indices, 0-based (params.f90:42-47 is 1-based) */
enum { RH = 0, MX = 1, MY = 2, MZ = 3, EN = 4, PXX = 5, PYY = 6, PZZ = 7, PXY = 8, PXZ = 9, PYZ = 10 };

struct orc_ctx {
    orc_params p;
    int nx, ny, nz, nb, iquad, nedge, nface, npg, nfe, npge, nslim, ibitri;
    /* basis index map, 1-based as in initialize.f90:126-194 */
    int kx, ky, kz, kyz, kzx, kxy, kxyz, kxx, kyy, kzz, kyzz, kzxx, kxyy;
    int kyyz, kzzx, kxxy, kyyzz, kzzxx, kxxyy, kyzxx, kzxyy, kxyzz;
    int kxyyzz, kyzzxx, kzxxyy, kxxyyzz, kxxx, kyyy, kzzz;
    double cbasis[NBT + 1];          /* 1-based */
    double xquad[20], wgt1d[5], wgt2d[30], wgt3d[100];
    /* tables [row][basis 1..30] stored as row*(NBT+1)+b */
    double *bfvals_int, *bfvals_xp, *bfvals_xm, *bfvals_yp, *bfvals_ym, *bfvals_zp, *bfvals_zm;
    double *bf_faces, *bval_int_wgt;
    double dx, dy, dz, dxi, dyi, dzi, cflm, aindm1;
    double c1d3, c2d3, c4d3;
    double P_floor;
    /* field work arrays */
    double *flux_x, *flux_y, *flux_z, *glflux_r, *source_r, *integral_r;
    /* trace arrays boundary.f90:735-740: Qxlo_int(ny,nz,nface,nQ) etc. */
    double *Qxlo_int, *Qxhi_int, *Qxlo_ext, *Qxhi_ext;
    double *Qylo_int, *Qyhi_int, *Qylo_ext, *Qyhi_ext;
    double *Qzlo_int, *Qzhi_int, *Qzlo_ext, *Qzhi_ext;
    double timers[6];
    unsigned long long noise_step;
    int noise_stage;
    int nonfinite;
};

#define TB(tab, row, b) ((tab)[(size_t)(row) * (NBT + 1) + (b)])
#define QI(c, i, j, k, v, b) ((size_t)(i) + (size_t)(c)->nx * ((j) + (size_t)(c)->ny * ((k) + (size_t)(c)->nz * ((v) + (size_t)NQ * (b)))))

static double wtime(void) {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

/* ---------------------------------------------------------------------------
 * Discretisation setup
 * ------------------------------------------------------------------------- */

/* initialize.f90:88-99 */
static int set_ibitri(int iquad, int nbasis) {
    int r = 0;
    if (iquad == 2 && nbasis == 4) r = 0;
    if (iquad == 3 && nbasis == 10) r = 0;
    if (iquad == 4 && nbasis == 20) r = 0;
    if (iquad == 2 && nbasis == 8) r = 1;
    if (iquad == 3 && nbasis == 27) r = 1;
    if (iquad == 4 && nbasis == 64) r = 1;
    return r;
}

/* initialize.f90:104-122 (identical for both ibitri) */
static double set_cflm(int iquad) {
    if (iquad == 2) return 0.14;
    if (iquad == 3) return 0.08;
    if (iquad == 4) return 0.05;
    return 0.14;
}

/* initialize.f90:126-194 */
static void set_basis_function_flags(orc_ctx *c) {
    int ib = c->ibitri, klim = 0;
    c->kx = 2; c->ky = 3; c->kz = 4; c->kyz = 5; c->kzx = 6; c->kxy = 7;
    if (ib == 0) klim = c->kxy;
    if (ib == 1) { c->kxyz = 8; klim = c->kxyz; }
    c->kxx = klim + 1; c->kyy = klim + 2; c->kzz = klim + 3;
    if (ib == 0) { c->kxyz = klim + 4; klim = c->kxyz; }
    if (ib == 1) klim = c->kzz;
    c->kyzz = klim + 1; c->kzxx = klim + 2; c->kxyy = klim + 3;
    c->kyyz = klim + 4; c->kzzx = klim + 5; c->kxxy = klim + 6;
    if (ib == 1) klim = c->kxxy;
    if (ib == 0) { c->kxxx = klim + 7; c->kyyy = klim + 8; c->kzzz = klim + 9; klim = c->kzzz; }
    c->kyyzz = klim + 1; c->kzzxx = klim + 2; c->kxxyy = klim + 3;
    c->kyzxx = klim + 4; c->kzxyy = klim + 5; c->kxyzz = klim + 6;
    c->kxyyzz = klim + 7; c->kyzzxx = klim + 8; c->kzxxyy = klim + 9; c->kxxyyzz = klim + 10;
    if (ib == 1) { c->kxxx = klim + 11; c->kyyy = klim + 12; c->kzzz = klim + 13; }
}

static void set_range(double *a, int lo, int hi, double v) {
    for (int i = lo; i <= hi; ++i) a[i] = v;
}

/* initialize.f90:199-220 */
static void set_cbasis_3D(orc_ctx *c) {
    double *cb = c->cbasis;
    memset(cb, 0, sizeof(c->cbasis));
    cb[1] = 1.;
    set_range(cb, c->kx, c->kz, 3.);
    set_range(cb, c->kyz, c->kxy, 9.);
    cb[c->kxyz] = 27.;
    set_range(cb, c->kxx, c->kzz, 5.);
    set_range(cb, c->kyzz, c->kxyy, 15.);
    set_range(cb, c->kyyz, c->kxxy, 15.);
    set_range(cb, c->kyyzz, c->kxxyy, 25.);
    set_range(cb, c->kyzxx, c->kxyzz, 45.);
    set_range(cb, c->kxyyzz, c->kzxxyy, 75.);
    cb[c->kxxyyzz] = 125.;
    set_range(cb, c->kxxx, c->kzzz, 7.);
}

static void set_xquad(orc_ctx *c) {
    double c15d5 = sqrt(15.) / 5., c1dsq3 = 1. / sqrt(3.);
    double xq4p = sqrt(525. + 70. * sqrt(30.)) / 35.;
    double xq4m = sqrt(525. - 70. * sqrt(30.)) / 35.;
    if (c->iquad == 2) { c->xquad[1] = -c1dsq3; c->xquad[2] = c1dsq3; }
    if (c->iquad == 3) { c->xquad[1] = -c15d5; c->xquad[2] = 0.; c->xquad[3] = c15d5; }
    if (c->iquad == 4) { c->xquad[1] = -xq4p; c->xquad[2] = -xq4m; c->xquad[3] = xq4m; c->xquad[4] = xq4p; }
}

/* products of the 1-D families for one row of a table (the product lines of
 * basis_funcs.f90:295-341 and the face/limiter analogues) */
static void set_products(const orc_ctx *c, double *t, int row) {
#define T_(b) TB(t, row, (b))
    T_(c->kyyz) = T_(c->kyy) * T_(c->kz);
    T_(c->kyzz) = T_(c->ky) * T_(c->kzz);
    T_(c->kzzx) = T_(c->kzz) * T_(c->kx);
    T_(c->kzxx) = T_(c->kz) * T_(c->kxx);
    T_(c->kxxy) = T_(c->kxx) * T_(c->ky);
    T_(c->kxyy) = T_(c->kx) * T_(c->kyy);
    T_(c->kyyzz) = T_(c->kyy) * T_(c->kzz);
    T_(c->kzzxx) = T_(c->kzz) * T_(c->kxx);
    T_(c->kxxyy) = T_(c->kxx) * T_(c->kyy);
    T_(c->kyzxx) = T_(c->kyz) * T_(c->kxx);
    T_(c->kzxyy) = T_(c->kzx) * T_(c->kyy);
    T_(c->kxyzz) = T_(c->kxy) * T_(c->kzz);
    T_(c->kxyyzz) = T_(c->kx) * T_(c->kyy) * T_(c->kzz);
    T_(c->kyzzxx) = T_(c->ky) * T_(c->kzz) * T_(c->kxx);
    T_(c->kzxxyy) = T_(c->kz) * T_(c->kxx) * T_(c->kyy);
    /* the reference forms this one as x*P2(y)*P2(z) (basis_funcs.f90:341) */
    T_(c->kxxyyzz) = T_(c->kx) * T_(c->kyy) * T_(c->kzz);
#undef T_
}

/* basis_funcs.f90:265-343 set_internal_vals_3D */
static void set_internal_vals_3D(orc_ctx *c) {
    int ne = c->nedge, nf = c->nface, npg = c->npg;
    double *t = c->bfvals_int;
    if (c->iquad == 1) {
        TB(t, 0, 1) = 1.; TB(t, 0, c->kx) = 0.; TB(t, 0, c->ky) = 0.; TB(t, 0, c->kz) = 0.;
    }
    if (c->iquad > 1) {
        for (int g = 0; g < npg; ++g) TB(t, g, 1) = 1.;
        for (int i = 1; i <= ne; ++i)
            for (int m = 1; m <= ne; ++m) {
                TB(t, (i - 1) * ne + m - 1, c->ky) = c->xquad[i];
                TB(t, (i - 1) * ne + m - 1, c->kz) = c->xquad[m];
            }
        for (int i = 1; i <= ne; ++i)
            for (int r = 0; r < nf; ++r) {
                TB(t, (i - 1) * nf + r, c->kx) = c->xquad[i];
                TB(t, (i - 1) * nf + r, c->ky) = TB(t, r, c->ky);
                TB(t, (i - 1) * nf + r, c->kz) = TB(t, r, c->kz);
            }
    }
    for (int g = 0; g < npg; ++g) {
        for (int i = 0; i <= 2; ++i) {
            double s = TB(t, g, c->kx + i);
            TB(t, g, c->kxx + i) = 1.5 * (s * s) - 0.5;
        }
        TB(t, g, c->kyz) = TB(t, g, c->ky) * TB(t, g, c->kz);
        TB(t, g, c->kzx) = TB(t, g, c->kz) * TB(t, g, c->kx);
        TB(t, g, c->kxy) = TB(t, g, c->kx) * TB(t, g, c->ky);
        TB(t, g, c->kxyz) = TB(t, g, c->kx) * TB(t, g, c->ky) * TB(t, g, c->kz);
        set_products(c, t, g);
    }
}

static void flip(const orc_ctx *c, double *t, int b) {
    for (int r = 0; r < c->nface; ++r) TB(t, r, b) = -TB(t, r, b);
}

/* basis_funcs.f90:346-567 set_face_vals_3D */
static void set_face_vals_3D(orc_ctx *c) {
    int ne = c->nedge, nf = c->nface;
    double *zp = c->bfvals_zp, *yp = c->bfvals_yp, *xp = c->bfvals_xp;
    for (int r = 0; r < nf; ++r) TB(zp, r, 1) = 1.;
    if (c->iquad == 1) { TB(zp, 0, c->kx) = 0.; TB(zp, 0, c->ky) = 0.; }
    if (c->iquad > 1)
        for (int i = 1; i <= ne; ++i)
            for (int m = 1; m <= ne; ++m) {
                TB(zp, (i - 1) * ne + m - 1, c->kx) = c->xquad[m];
                TB(zp, (i - 1) * ne + m - 1, c->ky) = c->xquad[i];
            }
    for (int r = 0; r < nf; ++r) {
        TB(zp, r, c->kz) = 1.;
        TB(zp, r, c->kyz) = TB(zp, r, c->ky) * TB(zp, r, c->kz);
        TB(zp, r, c->kzx) = TB(zp, r, c->kz) * TB(zp, r, c->kx);
        TB(zp, r, c->kxy) = TB(zp, r, c->kx) * TB(zp, r, c->ky);
        TB(zp, r, c->kxyz) = TB(zp, r, c->kx) * TB(zp, r, c->ky) * TB(zp, r, c->kz);

        TB(yp, r, 1) = 1.;
        TB(yp, r, c->kx) = TB(zp, r, c->ky);
        TB(yp, r, c->ky) = 1.;
        TB(yp, r, c->kz) = TB(zp, r, c->kx);
        TB(yp, r, c->kyz) = TB(yp, r, c->ky) * TB(yp, r, c->kz);
        TB(yp, r, c->kzx) = TB(yp, r, c->kz) * TB(yp, r, c->kx);
        TB(yp, r, c->kxy) = TB(yp, r, c->kx) * TB(yp, r, c->ky);
        TB(yp, r, c->kxyz) = TB(yp, r, c->kx) * TB(yp, r, c->ky) * TB(yp, r, c->kz);

        TB(xp, r, 1) = 1.;
        TB(xp, r, c->kx) = 1.;
        TB(xp, r, c->ky) = TB(zp, r, c->kx);
        TB(xp, r, c->kz) = TB(zp, r, c->ky);
        TB(xp, r, c->kyz) = TB(xp, r, c->ky) * TB(xp, r, c->kz);
        TB(xp, r, c->kzx) = TB(xp, r, c->kz) * TB(xp, r, c->kx);
        TB(xp, r, c->kxy) = TB(xp, r, c->kx) * TB(xp, r, c->ky);
        TB(xp, r, c->kxyz) = TB(xp, r, c->kx) * TB(xp, r, c->ky) * TB(xp, r, c->kz);

        for (int i = 0; i <= 2; ++i) {
            double s;
            s = TB(xp, r, c->kx + i); TB(xp, r, c->kxx + i) = 1.5 * (s * s) - 0.5;
            s = TB(yp, r, c->kx + i); TB(yp, r, c->kxx + i) = 1.5 * (s * s) - 0.5;
            s = TB(zp, r, c->kx + i); TB(zp, r, c->kxx + i) = 1.5 * (s * s) - 0.5;
        }
        set_products(c, xp, r);
        set_products(c, yp, r);
        set_products(c, zp, r);
    }
    size_t tbytes = (size_t)nf * (NBT + 1) * sizeof(double);
    memcpy(c->bfvals_xm, xp, tbytes);
    flip(c, c->bfvals_xm, c->kx); flip(c, c->bfvals_xm, c->kzx); flip(c, c->bfvals_xm, c->kxy);
    flip(c, c->bfvals_xm, c->kxyz); flip(c, c->bfvals_xm, c->kzzx); flip(c, c->bfvals_xm, c->kxyy);
    flip(c, c->bfvals_xm, c->kzxyy); flip(c, c->bfvals_xm, c->kxyzz); flip(c, c->bfvals_xm, c->kxyyzz);
    memcpy(c->bfvals_ym, yp, tbytes);
    flip(c, c->bfvals_ym, c->ky); flip(c, c->bfvals_ym, c->kyz); flip(c, c->bfvals_ym, c->kxy);
    flip(c, c->bfvals_ym, c->kxyz); flip(c, c->bfvals_ym, c->kyzz); flip(c, c->bfvals_ym, c->kxxy);
    flip(c, c->bfvals_ym, c->kyzxx); flip(c, c->bfvals_ym, c->kxyzz); flip(c, c->bfvals_ym, c->kyzzxx);
    memcpy(c->bfvals_zm, zp, tbytes);
    flip(c, c->bfvals_zm, c->kz); flip(c, c->bfvals_zm, c->kyz); flip(c, c->bfvals_zm, c->kzx);
    flip(c, c->bfvals_zm, c->kxyz); flip(c, c->bfvals_zm, c->kyyz); flip(c, c->bfvals_zm, c->kzxx);
    flip(c, c->bfvals_zm, c->kyzxx); flip(c, c->bfvals_zm, c->kzxyy); flip(c, c->bfvals_zm, c->kzxxyy);

    /* bf_faces, basis_funcs.f90:527-565: rows xm, xp, ym, yp, zm, zp, interior */
    double *bf = c->bf_faces;
    const double *src[6] = {c->bfvals_xm, c->bfvals_xp, c->bfvals_ym, c->bfvals_yp, c->bfvals_zm, c->bfvals_zp};
    for (int r = 0; r < c->nslim; ++r) TB(bf, r, 1) = 1.;
    for (int b = c->kx; b <= c->kz; ++b) {
        for (int f = 0; f < 6; ++f)
            for (int r = 0; r < nf; ++r) TB(bf, f * nf + r, b) = TB(src[f], r, b);
        for (int g = 0; g < c->npg; ++g) TB(bf, 6 * nf + g, b) = TB(c->bfvals_int, g, b);
    }
    for (int r = 0; r < c->nslim; ++r) {
        TB(bf, r, c->kyz) = TB(bf, r, c->ky) * TB(bf, r, c->kz);
        TB(bf, r, c->kzx) = TB(bf, r, c->kz) * TB(bf, r, c->kx);
        TB(bf, r, c->kxy) = TB(bf, r, c->kx) * TB(bf, r, c->ky);
        TB(bf, r, c->kxyz) = TB(bf, r, c->kx) * TB(bf, r, c->ky) * TB(bf, r, c->kz);
        for (int i = 0; i <= 2; ++i) {
            double s = TB(bf, r, c->kx + i);
            TB(bf, r, c->kxx + i) = 1.5 * (s * s) - 0.5;
        }
        set_products(c, bf, r);
    }
}

/* basis_funcs.f90:570-627 set_weights_3D */
static void set_weights_3D(orc_ctx *c) {
    int ne = c->nedge;
    double wq4p = (18. + sqrt(30.)) / 36., wq4m = (18. - sqrt(30.)) / 36.;
    if (c->iquad == 1) c->wgt1d[1] = 2.;
    if (c->iquad == 2) { c->wgt1d[1] = 1.; c->wgt1d[2] = 1.; }
    if (c->iquad == 3) { c->wgt1d[1] = 5. / 9.; c->wgt1d[2] = 8. / 9.; c->wgt1d[3] = 5. / 9.; }
    if (c->iquad == 4) { c->wgt1d[1] = wq4m; c->wgt1d[2] = wq4p; c->wgt1d[3] = wq4p; c->wgt1d[4] = wq4m; }
    if (c->iquad == 1) c->wgt2d[1] = 4.;
    if (c->iquad == 2) for (int i = 1; i <= 4; ++i) c->wgt2d[i] = 1.;
    if (c->iquad >= 3)
        for (int i = 1; i <= ne; ++i)
            for (int m = 1; m <= ne; ++m) c->wgt2d[(i - 1) * ne + m] = c->wgt1d[m] * c->wgt1d[i];
    if (c->iquad == 1) c->wgt3d[1] = 8.;
    if (c->iquad == 2) for (int i = 1; i <= 8; ++i) c->wgt3d[i] = 1.;
    if (c->iquad >= 3)
        for (int i = 1; i <= ne; ++i)
            for (int r = 1; r <= c->nface; ++r) c->wgt3d[(i - 1) * c->nface + r] = c->wgt2d[r] * c->wgt1d[i];
}

/* ---------------------------------------------------------------------------
 * Context
 * ------------------------------------------------------------------------- */

orc_ctx *orc_create(const orc_params *p) {
    orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
    if (!c) return NULL;
    c->p = *p;
    c->nx = p->nx; c->ny = p->ny; c->nz = p->nz;
    c->nb = p->nbasis; c->iquad = p->iquad;
    c->nedge = c->iquad; c->nface = c->iquad * c->iquad; c->npg = c->nface * c->iquad;
    c->nfe = 2 * c->nface; c->npge = 6 * c->nface; c->nslim = c->npg + 6 * c->nface;
    c->ibitri = set_ibitri(c->iquad, c->nb);
    set_basis_function_flags(c);
    set_cbasis_3D(c);
    c->cflm = p->cflm > 0 ? p->cflm : set_cflm(c->iquad);
    c->aindm1 = p->aindex - 1.;
    c->c1d3 = 1. / 3.; c->c2d3 = 2. / 3.; c->c4d3 = 4. / 3.;
    c->P_floor = p->T_floor * p->rh_floor;

    /* initialize.f90:298-327 (one rank) */
    c->dxi = (double)c->nx / p->lx;
    c->dyi = (double)c->ny / p->ly;
    c->dzi = (double)c->nz / p->lz;
    c->dx = 1. / c->dxi; c->dy = 1. / c->dyi; c->dz = 1. / c->dzi;

    size_t rb = (size_t)(NBT + 1) * sizeof(double);
    c->bfvals_int = (double *)calloc((size_t)c->npg, rb);
    c->bval_int_wgt = (double *)calloc((size_t)c->npg, rb);
    c->bfvals_xp = (double *)calloc((size_t)c->nface, rb);
    c->bfvals_xm = (double *)calloc((size_t)c->nface, rb);
    c->bfvals_yp = (double *)calloc((size_t)c->nface, rb);
    c->bfvals_ym = (double *)calloc((size_t)c->nface, rb);
    c->bfvals_zp = (double *)calloc((size_t)c->nface, rb);
    c->bfvals_zm = (double *)calloc((size_t)c->nface, rb);
    c->bf_faces = (double *)calloc((size_t)c->nslim, rb);
    set_xquad(c);
    set_internal_vals_3D(c);
    set_face_vals_3D(c);
    set_weights_3D(c);
    /* initialize.f90:366-370 */
    for (int b = 1; b <= c->nb; ++b)
        for (int g = 0; g < c->npg; ++g) TB(c->bval_int_wgt, g, b) = c->wgt3d[g + 1] * TB(c->bfvals_int, g, b);

    size_t nc = (size_t)c->nx * c->ny * c->nz;
    size_t nf = (size_t)c->nface;
    c->flux_x = (double *)calloc(nf * (c->nx + 1) * c->ny * c->nz * NQ, sizeof(double));
    c->flux_y = (double *)calloc(nf * c->nx * (c->ny + 1) * c->nz * NQ, sizeof(double));
    c->flux_z = (double *)calloc(nf * c->nx * c->ny * (c->nz + 1) * NQ, sizeof(double));
    c->glflux_r = (double *)calloc(nc * NQ * c->nb, sizeof(double));
    c->source_r = (double *)calloc(nc * NQ * c->nb, sizeof(double));
    c->integral_r = (double *)calloc(nc * NQ * c->nb, sizeof(double));
    size_t sx = (size_t)c->ny * c->nz * nf * NQ, sy = (size_t)c->nx * c->nz * nf * NQ, sz = (size_t)c->nx * c->ny * nf * NQ;
    c->Qxlo_int = calloc(sx, 8); c->Qxhi_int = calloc(sx, 8); c->Qxlo_ext = calloc(sx, 8); c->Qxhi_ext = calloc(sx, 8);
    c->Qylo_int = calloc(sy, 8); c->Qyhi_int = calloc(sy, 8); c->Qylo_ext = calloc(sy, 8); c->Qyhi_ext = calloc(sy, 8);
    c->Qzlo_int = calloc(sz, 8); c->Qzhi_int = calloc(sz, 8); c->Qzlo_ext = calloc(sz, 8); c->Qzhi_ext = calloc(sz, 8);
    return c;
}

void orc_destroy(orc_ctx *c) {
    if (!c) return;
    free(c->bfvals_int); free(c->bval_int_wgt); free(c->bfvals_xp); free(c->bfvals_xm);
    free(c->bfvals_yp); free(c->bfvals_ym); free(c->bfvals_zp); free(c->bfvals_zm); free(c->bf_faces);
    free(c->flux_x); free(c->flux_y); free(c->flux_z); free(c->glflux_r); free(c->source_r); free(c->integral_r);
    free(c->Qxlo_int); free(c->Qxhi_int); free(c->Qxlo_ext); free(c->Qxhi_ext);
    free(c->Qylo_int); free(c->Qyhi_int); free(c->Qylo_ext); free(c->Qyhi_ext);
    free(c->Qzlo_int); free(c->Qzhi_int); free(c->Qzlo_ext); free(c->Qzhi_ext);
    free(c);
}

long orc_qsize(const orc_ctx *c) { return (long)c->nx * c->ny * c->nz * NQ * c->nb; }
double orc_cflm(const orc_ctx *c) { return c->cflm; }

int orc_get_kindex(const orc_ctx *c, int *o) {
    int v[29] = {c->kx, c->ky, c->kz, c->kyz, c->kzx, c->kxy, c->kxyz, c->kxx, c->kyy, c->kzz,
                 c->kyzz, c->kzxx, c->kxyy, c->kyyz, c->kzzx, c->kxxy, c->kyyzz, c->kzzxx, c->kxxyy,
                 c->kyzxx, c->kzxyy, c->kxyzz, c->kxyyzz, c->kyzzxx, c->kzxxyy, c->kxxyyzz,
                 c->kxxx, c->kyyy, c->kzzz};
    for (int i = 0; i < 29; ++i) o[i] = v[i];
    return 29;
}

int orc_get_table(const orc_ctx *c, const char *name, double *out, int maxn) {
    const double *t = NULL;
    int rows = 0;
    if (!strcmp(name, "int")) { t = c->bfvals_int; rows = c->npg; }
    else if (!strcmp(name, "xp")) { t = c->bfvals_xp; rows = c->nface; }
    else if (!strcmp(name, "xm")) { t = c->bfvals_xm; rows = c->nface; }
    else if (!strcmp(name, "yp")) { t = c->bfvals_yp; rows = c->nface; }
    else if (!strcmp(name, "ym")) { t = c->bfvals_ym; rows = c->nface; }
    else if (!strcmp(name, "zp")) { t = c->bfvals_zp; rows = c->nface; }
    else if (!strcmp(name, "zm")) { t = c->bfvals_zm; rows = c->nface; }
    else if (!strcmp(name, "faces")) { t = c->bf_faces; rows = c->nslim; }
    else if (!strcmp(name, "cbasis")) { for (int b = 0; b < NBT && b < maxn; ++b) out[b] = c->cbasis[b + 1]; return NBT; }
    else if (!strcmp(name, "wgt3d")) { for (int g = 0; g < c->npg && g < maxn; ++g) out[g] = c->wgt3d[g + 1]; return c->npg; }
    else if (!strcmp(name, "wgt2d")) { for (int g = 0; g < c->nface && g < maxn; ++g) out[g] = c->wgt2d[g + 1]; return c->nface; }
    else return -1;
    int n = 0;
    for (int r = 0; r < rows; ++r)
        for (int b = 1; b <= NBT; ++b) {
            if (n < maxn) out[n] = TB(t, r, b);
            ++n;
        }
    return n;
}

/* ---------------------------------------------------------------------------
 * Stochastic stress: random.f90:106-145 with the reference's MKL MCG31 stream
 * replaced by counter-based Philox-4x32-10 (philox_ref.h).  The counter is
 * (call kind, site, point, step/stage); the same counter scheme is used by
 * the CUDA kernels so a run with noise on is reproducible bit for bit in the
 * random inputs.
 * ------------------------------------------------------------------------- */
enum { NOISE_FACE_X = 0, NOISE_FACE_Y = 1, NOISE_FACE_Z = 2, NOISE_INT_X = 3, NOISE_INT_Y = 4, NOISE_INT_Z = 5 };

static void stress_at(const orc_ctx *c, int kind, unsigned long long site, int pt, double S[6]) {
    double G[6];
    hermes_philox_normals6(c->p.seed, c->noise_step, (unsigned)c->noise_stage, (unsigned)kind, site, (unsigned)pt, G);
    /* random.f90:124-141 (amplitudes eta_sd, zeta_sd already carry 1/sqrt(dV dt)):
     * the diagonal G_ii and the symmetrised off-diagonal sqrt(1/2) (G_ij + G_ji)
     * of an iid N(0,1) matrix are six iid N(0,1) values, drawn directly */
    double Gxx = G[0], Gyy = G[1], Gzz = G[2];
    double Gxy = G[3], Gxz = G[4], Gyz = G[5];
    double trG = Gxx + Gyy + Gzz, trGd3 = trG / 3.0, trGz = c->p.zeta_sd * trG;
    S[0] = c->p.eta_sd * (Gxx - trGd3) + trGz;  /* Sxx */
    S[1] = c->p.eta_sd * (Gyy - trGd3) + trGz;  /* Syy */
    S[2] = c->p.eta_sd * (Gzz - trGd3) + trGz;  /* Szz */
    S[3] = c->p.eta_sd * Gxy;                   /* Sxy */
    S[4] = c->p.eta_sd * Gxz;                   /* Sxz */
    S[5] = c->p.eta_sd * Gyz;                   /* Syz */
}

/* ---------------------------------------------------------------------------
 * flux.f90:23-193 flux_calc_pnts_r.  Qp, fp are (npnts, nQ) column-major.
 * noise_kind < 0: no stochastic stress (the reference default, llns off).
 * ------------------------------------------------------------------------- */
static void flux_calc_pnts_r(const orc_ctx *c, const double *Qp, double *fp, int ixyz, int npnts,
                             int noise_kind, unsigned long long noise_site) {
    const double aindm1 = c->aindm1, c1d3 = c->c1d3;
    const double colvis = c->p.colvis;
    const double c2d3cv = c->c2d3 * colvis, c4d3cv = c->c4d3 * colvis;
    const int ivis = c->p.ivis;
    for (int ife = 0; ife < npnts; ++ife) {
#define QP(v) Qp[(size_t)(v) * npnts + ife]
#define FP(v) fp[(size_t)(v) * npnts + ife]
        double dn = QP(RH), M_x = QP(MX), M_y = QP(MY), M_z = QP(MZ), Ener = QP(EN);
        double P_xx = QP(PXX), P_yy = QP(PYY), P_zz = QP(PZZ), P_xy = QP(PXY), P_xz = QP(PXZ), P_yz = QP(PYZ);
        double dni = 1. / dn;
        double vx = M_x * dni, vy = M_y * dni, vz = M_z * dni;
        double smsq = M_x * M_x + M_y * M_y + M_z * M_z;
        double P = aindm1 * (Ener - 0.5 * dni * smsq);
        double P_10 = c1d3 * (P_xx + P_yy + P_zz - dni * smsq);
        if (c->p.ieos == 2) P = c->p.P_1 * (pow(dn, 7.2) - 1.) + c->p.P_base + P;
        if (P < c->P_floor) P = c->P_floor;
        if (P_10 < c->P_floor) P_10 = c->P_floor;
        double P_5 = P;
        double Sxx = 0, Syy = 0, Szz = 0, Sxy = 0, Sxz = 0, Syz = 0;
        if (noise_kind >= 0) {
            double S[6];
            stress_at(c, noise_kind, noise_site, ife, S);
            Sxx = S[0]; Syy = S[1]; Szz = S[2]; Sxy = S[3]; Sxz = S[4]; Syz = S[5];
        }
        switch (ixyz) {
        case 1:
            FP(RH) = M_x;
            if (ivis == 0 || ivis == 1) {
                FP(MX) = M_x * vx + P + P_xx - Sxx;
                FP(MY) = M_y * vx + P_xy - Sxy;
                FP(MZ) = M_z * vx + P_xz - Sxz;
            } else {
                FP(MX) = P_xx - P_10 + P_5;
                FP(MY) = P_xy;
                FP(MZ) = P_xz;
            }
            FP(EN) = (Ener + P) * vx + (P_xx - Sxx) * vx + (P_xy - Sxy) * vy + (P_xz - Sxz) * vz;
            /* Grad closure (ivis 3): dg_3D_hydro_bitri_ten_moment.f90:969 */
            if (ivis == 3) FP(EN) = (Ener + P) * vx;
            if (ivis == 0 || ivis == 1) {
                FP(PXX) = c4d3cv * vx; FP(PYY) = -c2d3cv * vx; FP(PZZ) = -c2d3cv * vx;
                FP(PXY) = colvis * vy; FP(PXZ) = colvis * vz; FP(PYZ) = 0;
            } else {
                FP(PXX) = vx * (3 * P_xx - 2 * vx * M_x);
                FP(PYY) = 2 * vy * (P_xy - vy * M_x) + vx * P_yy;
                FP(PZZ) = 2 * vz * (P_xz - vz * M_x) + vx * P_zz;
                FP(PXY) = 2 * vx * (P_xy - vy * M_x) + vy * P_xx;
                FP(PXZ) = 2 * vx * (P_xz - vz * M_x) + vz * P_xx;
                FP(PYZ) = vx * P_yz + vy * P_xz + vz * P_xy - 2 * vy * vz * M_x;
            }
            break;
        case 2:
            FP(RH) = M_y;
            if (ivis == 0 || ivis == 1) {
                FP(MX) = M_x * vy + P_xy - Sxy;
                FP(MY) = M_y * vy + P + P_yy - Syy;
                FP(MZ) = M_z * vy + P_yz - Syz;
            } else {
                FP(MX) = P_xy;
                FP(MY) = P_yy - P_10 + P_5;
                FP(MZ) = P_yz;
            }
            FP(EN) = (Ener + P) * vy + (P_yy - Syy) * vy + (P_xy - Sxy) * vx + (P_yz - Syz) * vz;
            /* Grad closure (ivis 3): dg_3D_hydro_bitri_ten_moment.f90:969 */
            if (ivis == 3) FP(EN) = (Ener + P) * vy;
            if (ivis == 0 || ivis == 1) {
                FP(PXX) = -c2d3cv * vy; FP(PYY) = c4d3cv * vy; FP(PZZ) = -c2d3cv * vy;
                FP(PXY) = colvis * vx; FP(PXZ) = 0; FP(PYZ) = colvis * vz;
            } else {
                FP(PXX) = 2 * vx * (P_xy - vx * M_y) + vy * P_xx;
                FP(PYY) = vy * (3 * P_yy - 2 * vy * M_y);
                FP(PZZ) = 2 * vz * (P_yz - vz * M_y) + vy * P_zz;
                FP(PXY) = 2 * vy * (P_xy - vx * M_y) + vx * P_yy;
                FP(PXZ) = vx * P_yz + vy * P_xz + vz * P_xy - 2 * vx * vz * M_y;
                FP(PYZ) = 2 * vy * (P_yz - vz * M_y) + vz * P_yy;
            }
            break;
        default:
            FP(RH) = M_z;
            if (ivis == 0 || ivis == 1) {
                FP(MX) = M_x * vz + P_xz - Sxz;
                FP(MY) = M_y * vz + P_yz - Syz;
                FP(MZ) = M_z * vz + P + P_zz - Szz;
            } else {
                FP(MX) = P_xz;
                FP(MY) = P_yz;
                FP(MZ) = P_zz - P_10 + P_5;
            }
            FP(EN) = (Ener + P) * vz + (P_zz - Szz) * vz + (P_xz - Sxz) * vx + (P_yz - Syz) * vy;
            /* Grad closure (ivis 3): dg_3D_hydro_bitri_ten_moment.f90:969 */
            if (ivis == 3) FP(EN) = (Ener + P) * vz;
            if (ivis == 0 || ivis == 1) {
                FP(PXX) = -c2d3cv * vz; FP(PYY) = -c2d3cv * vz; FP(PZZ) = c4d3cv * vz;
                FP(PXY) = 0; FP(PXZ) = colvis * vx; FP(PYZ) = colvis * vy;
            } else {
                FP(PXX) = 2 * vx * (P_xz - vx * M_z) + vz * P_xx;
                FP(PYY) = 2 * vy * (P_yz - vy * M_z) + vz * P_yy;
                FP(PZZ) = vz * (3 * P_zz - 2 * vz * M_z);
                FP(PXY) = vx * P_yz + vy * P_xz + vz * P_xy - 2 * vx * vy * M_z;
                FP(PXZ) = 2 * vz * (P_xz - vx * M_z) + vx * P_zz;
                FP(PYZ) = 2 * vz * (P_yz - vy * M_z) + vy * P_zz;
            }
            break;
        }
#undef QP
#undef FP
    }
}

/* flux.f90:1029-1072 cfcal */
static double cfcal(const orc_ctx *c, const double *Qcf, int cases) {
    double dn = Qcf[RH], dni = 1. / dn;
    double vx = Qcf[MX] * dni, vy = Qcf[MY] * dni, vz = Qcf[MZ] * dni;
    double P = 0., cs = 0.;
    if (c->p.ivis == 0 || c->p.ivis == 1) P = c->aindm1 * (Qcf[EN] - 0.5 * dn * (vx * vx + vy * vy + vz * vz));
    else P = c->c1d3 * (Qcf[PXX] + Qcf[PYY] + Qcf[PZZ] - dn * (vx * vx + vy * vy + vz * vz));
    if (c->p.ieos == 1) cs = sqrt(c->p.aindex * P * dni);
    else cs = sqrt(7.2 * c->p.P_1 * pow(dn, 6.2));
    if (cases == 1) return fabs(vx) + cs;
    if (cases == 2) return fabs(vy) + cs;
    return fabs(vz) + cs;
}

/* flux.f90:466-647 flux_hllc (ibatten = 0).  Qlr, flr are (nfe, nQ);
 * fhllc is (nface, 5) in natural variable order. */
static void flux_hllc(const orc_ctx *c, const double *Qlr, const double *flr, double *fhllc, int ixyz) {
    const int nf = c->nface, nfe = c->nfe;
    int iparr, iperp1, iperp2;
    if (ixyz == 1) { iparr = MX; iperp1 = MY; iperp2 = MZ; }
    else if (ixyz == 2) { iparr = MY; iperp1 = MZ; iperp2 = MX; }
    else { iparr = MZ; iperp1 = MX; iperp2 = MY; }
    int ivar[5] = {RH, iparr, iperp1, iperp2, EN};
    double rhov[32], vlr[32][3], qsq[32], plr[32], cslr[32], qslr[32], s_lr[32];
    double sm_num[16], sm_den[16], s_m[16], pstar[16];
    double aindex = c->p.aindex, aindm1 = c->aindm1;
    double rho_i = 0.;
#define QL(k, v) Qlr[(size_t)(v) * nfe + (k)]
#define FL(k, v) flr[(size_t)(v) * nfe + (k)]
    for (int k = 0; k < nfe; ++k) {
        rhov[k] = QL(k, RH);
        rho_i = 1.0 / rhov[k];
        vlr[k][0] = QL(k, iparr) * rho_i;
        vlr[k][1] = QL(k, iperp1) * rho_i;
        vlr[k][2] = QL(k, iperp2) * rho_i;
        qsq[k] = vlr[k][0] * vlr[k][0] + vlr[k][1] * vlr[k][1] + vlr[k][2] * vlr[k][2];
        plr[k] = aindm1 * (QL(k, EN) - 0.5 * rhov[k] * qsq[k]);
        if (c->p.ieos == 2) plr[k] = c->p.P_1 * (pow(rhov[k], 7.2) - 1.) + c->p.P_base + plr[k];
    }
    /* rho_i now holds the value of the last point: the reference's ieos-2
     * branch uses it for every point (flux.f90:533-534,570-571) */
    for (int k = 0; k < nf; ++k) {
        int k2 = k + nf;
        if (c->p.ieos == 2) {
            cslr[k] = vlr[k][0] - sqrt(7.2 * c->p.P_1 * pow(rhov[k], 6.2) + plr[k] * rho_i);
            cslr[k2] = vlr[k2][0] + sqrt(7.2 * c->p.P_1 * pow(rhov[k2], 6.2) + plr[k2] * rho_i);
        } else {
            cslr[k] = vlr[k][0] - sqrt(aindex * plr[k] / rhov[k]);
            cslr[k2] = vlr[k2][0] + sqrt(aindex * plr[k2] / rhov[k2]);
        }
    }
    for (int k = 0; k < nf; ++k) {
        int k2 = k + nf;
        if (c->p.ieos == 2) {
            qslr[k] = vlr[k2][0] - sqrt(7.2 * c->p.P_1 * pow(rhov[k2], 6.2) + plr[k2] * rho_i);
            qslr[k2] = vlr[k][0] + sqrt(7.2 * c->p.P_1 * pow(rhov[k], 6.2) + plr[k] * rho_i);
        } else {
            qslr[k] = vlr[k2][0] - sqrt(aindex * plr[k2] / rhov[k2]);
            qslr[k2] = vlr[k][0] + sqrt(aindex * plr[k] / rhov[k]);
        }
    }
    for (int k = 0; k < nf; ++k) {
        int k2 = k + nf;
        s_lr[k] = fmin(cslr[k], qslr[k]);
        s_lr[k2] = fmax(cslr[k2], qslr[k2]);
        sm_num[k] = rhov[k2] * vlr[k2][0] * (s_lr[k2] - vlr[k2][0]) - rhov[k] * vlr[k][0] * (s_lr[k] - vlr[k][0]);
        sm_num[k] = sm_num[k] + plr[k] - plr[k2];
        sm_den[k] = rhov[k2] * (s_lr[k2] - vlr[k2][0]) - rhov[k] * (s_lr[k] - vlr[k][0]);
    }
    for (int k = 0; k < nf; ++k)
        if (sm_den[k] == 0.0) sm_den[k] = c->p.rh_floor;
    for (int k = 0; k < nf; ++k) {
        s_m[k] = sm_num[k] / sm_den[k];
        pstar[k] = rhov[k] * (vlr[k][0] - s_lr[k]) * (vlr[k][0] - s_m[k]) + plr[k];
    }
    double fstar[32][5];
    for (int k = 0; k < nfe; ++k) {
        int i4 = k < nf ? k : k - nf;
        double den = s_lr[k] - s_m[i4];
        if (den == 0.0) den = c->p.rh_floor;
        double slrm_i = 1.0 / den;
        double sq_lr = s_lr[k] - vlr[k][0];
        double Qs[5];
        Qs[0] = rhov[k] * sq_lr * slrm_i;
        Qs[1] = (sq_lr * QL(k, iparr) + pstar[i4] - plr[k]) * slrm_i;
        Qs[2] = sq_lr * QL(k, iperp1) * slrm_i;
        Qs[3] = sq_lr * QL(k, iperp2) * slrm_i;
        Qs[4] = (sq_lr * QL(k, EN) - plr[k] * vlr[k][0] + pstar[i4] * s_m[i4]) * slrm_i;
        for (int e = 0; e < 5; ++e) fstar[k][e] = FL(k, ivar[e]) + s_lr[k] * (Qs[e] - QL(k, ivar[e]));
    }
    for (int i4 = 0; i4 < nf; ++i4) {
        double out[5];
        for (int e = 0; e < 5; ++e) out[e] = NAN; /* no branch taken only for NaN input */
        if (s_lr[i4] > 0.0)
            for (int e = 0; e < 5; ++e) out[e] = FL(i4, ivar[e]);
        if (s_lr[i4] <= 0.0 && 0.0 < s_m[i4])
            for (int e = 0; e < 5; ++e) out[e] = fstar[i4][e];
        if (s_m[i4] <= 0.0 && 0.0 <= s_lr[i4 + nf])
            for (int e = 0; e < 5; ++e) out[e] = fstar[i4 + nf][e];
        if (s_lr[i4 + nf] < 0.0)
            for (int e = 0; e < 5; ++e) out[e] = FL(i4 + nf, ivar[e]);
        /* fhllc(i4, ivar(e)) = out(e) */
        for (int e = 0; e < 5; ++e) fhllc[(size_t)ivar[e] * nf + i4] = out[e];
    }
#undef QL
#undef FL
}

/* Roe solver of the monolithic 10-moment code
 * (src/ces/10_moment/dg_3D_hydro_lqc_SEAN.f90:1614-1789, Eulderink-Mellema):
 * F = (F_L + F_R - dF)/2 for rh..en with dF from the Roe-averaged
 * eigensystem; kroe = 0 (keep the central/LLF flux) where the Roe sound speed
 * squared is <= 0.  Reproduces the reference's Roe enthalpy, whose pressure
 * term carries a factor 1/2 (:1676). */
static void flux_roe(const orc_ctx *c, const double *Qlr, const double *flr, double *froe, int *kroe, int ixyz) {
    const int nf = c->nface, nfe = c->nfe;
    int ip, i1, i2;
    if (ixyz == 1) { ip = MX; i1 = MY; i2 = MZ; }
    else if (ixyz == 2) { ip = MY; i1 = MZ; i2 = MX; }
    else { ip = MZ; i1 = MX; i2 = MY; }
    const double aindm1 = c->aindm1, cp = c->p.aindex / c->aindm1;
#define QL(k, v) Qlr[(size_t)(v) * nfe + (k)]
#define FL(k, v) flr[(size_t)(v) * nfe + (k)]
    for (int i9 = 0; i9 < nf; ++i9) {
        double skr[2], swr[2][4];
        kroe[i9] = 1;
        for (int j9 = 0; j9 < 2; ++j9) {
            int ilr = i9 + j9 * nf;
            double dnii = 1. / QL(ilr, RH);
            double v0 = QL(ilr, ip) * dnii, v1 = QL(ilr, i1) * dnii, v2 = QL(ilr, i2) * dnii;
            double vsq = v0 * v0 + v1 * v1 + v2 * v2;
            double Pri = aindm1 * (QL(ilr, EN) - 0.5 * QL(ilr, RH) * vsq);
            skr[j9] = sqrt(QL(ilr, RH));
            swr[j9][0] = skr[j9] * v0;
            swr[j9][1] = skr[j9] * v1;
            swr[j9][2] = skr[j9] * v2;
            swr[j9][3] = 0.5 * skr[j9] * (vsq + cp * Pri / QL(ilr, RH));
        }
        double Qri = 1. / QL(i9, RH);
        double delrho = QL(i9 + nf, RH) * Qri - 1.;
        double dele = (QL(i9 + nf, EN) - QL(i9, EN)) * Qri;
        double dm1 = (QL(i9 + nf, ip) - QL(i9, ip)) * Qri;
        double dm2 = (QL(i9 + nf, i1) - QL(i9, i1)) * Qri;
        double dm3 = (QL(i9 + nf, i2) - QL(i9, i2)) * Qri;
        double dwr[4];
        for (int j = 0; j < 4; ++j) dwr[j] = 0.5 * (swr[1][j] + swr[0][j]);
        double dsk = 0.5 * (skr[1] + skr[0]);
        double vc0 = dwr[0] / dsk, vc1 = dwr[1] / dsk, vc2 = dwr[2] / dsk, hc = dwr[3] / dsk;
        double vcsq = vc0 * vc0 + vc1 * vc1 + vc2 * vc2;
        double asq = aindm1 * (hc - 0.5 * vcsq);
        if (asq <= 0.0) kroe[i9] = 0;
        double sc9 = sqrt(asq);
        double lam[5] = {fabs(vc0 - sc9), fabs(vc0 + sc9), fabs(vc0), fabs(vc0), fabs(vc0)};
        /* evec[row][col]: rows density, energy, parallel, perp1, perp2 */
        double ev[5][5] = {{1., 1., 1., 0., 0.},
                           {hc - sc9 * vc0, hc + sc9 * vc0, 0.5 * vcsq, vc1, vc2},
                           {vc0 - sc9, vc0 + sc9, vc0, 0., 0.},
                           {vc1, vc1, vc1, 1., 0.},
                           {vc2, vc2, vc2, 0., 1.}};
        double ea2i = aindm1 / asq;
        double vcdel = vc0 * dm1 + vc1 * dm2 + vc2 * dm3 - dele;
        double a9e = 0.5 * ea2i * (0.5 * vcsq * delrho - vcdel);
        double sk9 = 0.5 * (dm1 - vc0 * delrho) / sc9;
        double a9[5] = {a9e - sk9, a9e + sk9, ea2i * ((hc - vcsq) * delrho + vcdel), dm2 - vc1 * delrho, dm3 - vc2 * delrho};
        double df[5];
        for (int r = 0; r < 5; ++r) {
            df[r] = 0.;
            for (int j = 0; j < 5; ++j) df[r] = df[r] + a9[j] * lam[j] * ev[r][j];
            df[r] = df[r] * QL(i9, RH);
        }
        froe[(size_t)RH * nf + i9] = 0.5 * (FL(i9, RH) + FL(i9 + nf, RH) - df[0]);
        froe[(size_t)EN * nf + i9] = 0.5 * (FL(i9, EN) + FL(i9 + nf, EN) - df[1]);
        froe[(size_t)ip * nf + i9] = 0.5 * (FL(i9, ip) + FL(i9 + nf, ip) - df[2]);
        froe[(size_t)i1 * nf + i9] = 0.5 * (FL(i9, i1) + FL(i9 + nf, i1) - df[3]);
        froe[(size_t)i2 * nf + i9] = 0.5 * (FL(i9, i2) + FL(i9 + nf, i2) - df[4]);
    }
#undef QL
#undef FL
}

/* ---------------------------------------------------------------------------
 * Trace exchange and boundaries (prepare_step.f90:20-68, boundary.f90)
 * ------------------------------------------------------------------------- */
static double trace(const orc_ctx *c, const double *tab, int pnt, const double *Q, int i, int j, int k, int v) {
    double s = 0.;
    for (int b = 1; b <= c->nb; ++b) s += TB(tab, pnt, b) * Q[QI(c, i, j, k, v, b - 1)];
    return s;
}

/* index of a boundary trace array, e.g. Qxlo_int(j,k,ipnt,ieq) */
static inline size_t BI(int a, int na, int b, int nbb, int p, int nf, int v) {
    return (size_t)a + (size_t)na * (b + (size_t)nbb * (p + (size_t)nf * v));
}

/* boundary.f90:40-338: ghost trace from the interior trace for one face of
 * the domain.  lo = 1 for a low face.  mom = normal momentum index. */
static void apply_bc(const orc_ctx *c, int code, int lo, int mom, int na, int nbb, const double *qi, double *qe) {
    int nf = c->nface;
    if (code == ORC_BC_PERIODIC) return;
    for (int b = 0; b < nbb; ++b)
        for (int a = 0; a < na; ++a) {
            if (code == ORC_BC_OUTFLOW && mom == MX && !lo) {
                /* boundary.f90:246-282: the interior trace is never copied;
                 * only positive normal momentum of the stale ghost flips */
                for (int p = 0; p < nf; ++p) {
                    size_t ix = BI(a, na, b, nbb, p, nf, MX);
                    if (qe[ix] > 0.0) qe[ix] = -qi[ix];
                }
                continue;
            }
            for (int v = 0; v < NQ; ++v)
                for (int p = 0; p < nf; ++p) qe[BI(a, na, b, nbb, p, nf, v)] = qi[BI(a, na, b, nbb, p, nf, v)];
            if (code == ORC_BC_INFLOW && mom == MX && lo) {
                /* boundary.f90:568-612 x_bc_inflow with the profile of
                 * set_xlobc_inflow: yp = yc(j) - lyd, vx = 4 u yp (ly - yp)/ly^2 */
                const double ly = c->p.ly, lyd = -(ly / 2.0);
                const double yc = lyd + (a + 0.5) * (1.0 / (c->ny / ly));
                const double yp = yc - lyd;
                const double vx = 4 * c->p.inflow_u * yp * (ly - yp) / (ly * ly);
                const double den = c->p.inflow_rho, pres = c->p.inflow_p;
                for (int p = 0; p < nf; ++p) {
                    qe[BI(a, na, b, nbb, p, nf, RH)] = den;
                    qe[BI(a, na, b, nbb, p, nf, MX)] = den * vx;
                    qe[BI(a, na, b, nbb, p, nf, MY)] = 0.0;
                    qe[BI(a, na, b, nbb, p, nf, MZ)] = 0.0;
                    qe[BI(a, na, b, nbb, p, nf, EN)] = pres / (c->p.aindex - 1.0) + 0.5 * den * (vx * vx);
                }
            }
            if (code == ORC_BC_NOSLIP) {
                for (int v = MX; v <= MZ; ++v)
                    for (int p = 0; p < nf; ++p) qe[BI(a, na, b, nbb, p, nf, v)] = 0.0;
            } else if (code == ORC_BC_WALL) {
                for (int p = 0; p < nf; ++p) qe[BI(a, na, b, nbb, p, nf, mom)] = 0.0;
            } else if (code == ORC_BC_OUTFLOW) {
                if (lo) {
                    double mx = -INFINITY;
                    for (int p = 0; p < nf; ++p) mx = fmax(mx, qe[BI(a, na, b, nbb, p, nf, mom)]);
                    if (mx > 0.0)
                        for (int p = 0; p < nf; ++p) qe[BI(a, na, b, nbb, p, nf, mom)] = 0.0;
                } else {
                    double mn = INFINITY;
                    for (int p = 0; p < nf; ++p) mn = fmin(mn, qe[BI(a, na, b, nbb, p, nf, mom)]);
                    if (mn < 0.0)
                        for (int p = 0; p < nf; ++p) qe[BI(a, na, b, nbb, p, nf, mom)] = 0.0;
                }
            }
        }
}

static void exchange_and_bc(orc_ctx *c, const double *Q) {
    int nx = c->nx, ny = c->ny, nz = c->nz, nf = c->nface;
    for (int v = 0; v < NQ; ++v)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int p = 0; p < nf; ++p) {
                    c->Qxlo_int[BI(j, ny, k, nz, p, nf, v)] = trace(c, c->bfvals_xm, p, Q, 0, j, k, v);
                    c->Qxhi_int[BI(j, ny, k, nz, p, nf, v)] = trace(c, c->bfvals_xp, p, Q, nx - 1, j, k, v);
                }
    for (int v = 0; v < NQ; ++v)
        for (int k = 0; k < nz; ++k)
            for (int i = 0; i < nx; ++i)
                for (int p = 0; p < nf; ++p) {
                    c->Qylo_int[BI(i, nx, k, nz, p, nf, v)] = trace(c, c->bfvals_ym, p, Q, i, 0, k, v);
                    c->Qyhi_int[BI(i, nx, k, nz, p, nf, v)] = trace(c, c->bfvals_yp, p, Q, i, ny - 1, k, v);
                }
    for (int v = 0; v < NQ; ++v)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i)
                for (int p = 0; p < nf; ++p) {
                    c->Qzlo_int[BI(i, nx, j, ny, p, nf, v)] = trace(c, c->bfvals_zm, p, Q, i, j, 0, v);
                    c->Qzhi_int[BI(i, nx, j, ny, p, nf, v)] = trace(c, c->bfvals_zp, p, Q, i, j, nz - 1, v);
                }
    /* prepare_step.f90:75-179 on one rank: a periodic dimension (chosen by
     * the *hi* flag, initialize.f90:255-263) is a send to self */
    size_t sx = (size_t)ny * nz * nf * NQ, sy = (size_t)nx * nz * nf * NQ, sz = (size_t)nx * ny * nf * NQ;
    if (c->p.bc[1] == ORC_BC_PERIODIC) {
        memcpy(c->Qxlo_ext, c->Qxhi_int, sx * 8); memcpy(c->Qxhi_ext, c->Qxlo_int, sx * 8);
    }
    if (c->p.bc[3] == ORC_BC_PERIODIC) {
        memcpy(c->Qylo_ext, c->Qyhi_int, sy * 8); memcpy(c->Qyhi_ext, c->Qylo_int, sy * 8);
    }
    if (c->p.bc[5] == ORC_BC_PERIODIC) {
        memcpy(c->Qzlo_ext, c->Qzhi_int, sz * 8); memcpy(c->Qzhi_ext, c->Qzlo_int, sz * 8);
    }
    /* boundary.f90:748-782 apply_boundaries */
    apply_bc(c, c->p.bc[0], 1, MX, ny, nz, c->Qxlo_int, c->Qxlo_ext);
    apply_bc(c, c->p.bc[1], 0, MX, ny, nz, c->Qxhi_int, c->Qxhi_ext);
    apply_bc(c, c->p.bc[2], 1, MY, nx, nz, c->Qylo_int, c->Qylo_ext);
    apply_bc(c, c->p.bc[3], 0, MY, nx, nz, c->Qyhi_int, c->Qyhi_ext);
    apply_bc(c, c->p.bc[4], 1, MZ, nx, ny, c->Qzlo_int, c->Qzlo_ext);
    apply_bc(c, c->p.bc[5], 0, MZ, nx, ny, c->Qzhi_int, c->Qzhi_ext);
}

/* ---------------------------------------------------------------------------
 * flux.f90:197-450 calc_flux_x/y/z, written once for a direction d
 * ------------------------------------------------------------------------- */
static void calc_flux_dir(orc_ctx *c, const double *Q, int d) {
    const int nx = c->nx, ny = c->ny, nz = c->nz, nf = c->nface, nfe = c->nfe;
    const double *tp = d == 1 ? c->bfvals_xp : d == 2 ? c->bfvals_yp : c->bfvals_zp;
    const double *tm = d == 1 ? c->bfvals_xm : d == 2 ? c->bfvals_ym : c->bfvals_zm;
    double *flux = d == 1 ? c->flux_x : d == 2 ? c->flux_y : c->flux_z;
    const int fx = nx + (d == 1), fy = ny + (d == 2), fz = nz + (d == 3);
    const int noise = c->p.llns ? (NOISE_FACE_X + d - 1) : -1;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < fz; ++k)
        for (int j = 0; j < fy; ++j) {
            double Qf[32 * NQ], ff[32 * NQ], fh[16 * NQ], cw[32], cfr[16];
            for (int i = 0; i < fx; ++i) {
                int ci = i, cj = j, ck = k;       /* the cell on the high side */
                int li = i - (d == 1), lj = j - (d == 2), lk = k - (d == 3);  /* low side */
                int first = (d == 1 ? i == 0 : d == 2 ? j == 0 : k == 0);
                int last = (d == 1 ? i == nx : d == 2 ? j == ny : k == nz);
                for (int v = 0; v < NQ; ++v)
                    for (int p = 0; p < nf; ++p) {
                        double L, R;
                        if (!first) L = trace(c, tp, p, Q, li, lj, lk, v);
                        else if (d == 1) L = c->Qxlo_ext[BI(j, ny, k, nz, p, nf, v)];
                        else if (d == 2) L = c->Qylo_ext[BI(i, nx, k, nz, p, nf, v)];
                        else L = c->Qzlo_ext[BI(i, nx, j, ny, p, nf, v)];
                        if (!last) R = trace(c, tm, p, Q, ci, cj, ck, v);
                        else if (d == 1) R = c->Qxhi_ext[BI(j, ny, k, nz, p, nf, v)];
                        else if (d == 2) R = c->Qyhi_ext[BI(i, nx, k, nz, p, nf, v)];
                        else R = c->Qzhi_ext[BI(i, nx, j, ny, p, nf, v)];
                        Qf[v * nfe + p] = L;
                        Qf[v * nfe + p + nf] = R;
                    }
                /* noise site: face index on the grid of distinct faces; a
                 * direction periodic at both ends has n planes (the plane at
                 * n is the plane at 0, and gets the same noise) */
                unsigned long long site = 0;
                if (noise >= 0) {
                    int pd = c->p.bc[2 * (d - 1)] == ORC_BC_PERIODIC && c->p.bc[2 * (d - 1) + 1] == ORC_BC_PERIODIC;
                    int si = i, sj = j, sk = k, ex = fx, ey = fy;
                    if (pd && d == 1) { ex = nx; si = i % nx; }
                    if (pd && d == 2) { ey = ny; sj = j % ny; }
                    if (pd && d == 3) { sk = k % nz; }
                    site = (unsigned long long)si + (unsigned long long)ex * (sj + (unsigned long long)ey * sk);
                }
                flux_calc_pnts_r(c, Qf, ff, d, nfe, noise, site);
                for (int p = 0; p < nf; ++p) cfr[p] = 0.0;
                if (c->p.ivis >= 2) {   /* ivis 3: the monolith always applies LLF (ten_moment.f90:1131-1147) */
                    for (int p = 0; p < nfe; ++p) {
                        double qv[NQ];
                        for (int v = 0; v < NQ; ++v) qv[v] = Qf[v * nfe + p];
                        cw[p] = cfcal(c, qv, d);
                    }
                    for (int p = 0; p < nf; ++p) cfr[p] = fmax(cw[p], cw[p + nf]);
                }
                for (int v = 0; v < NQ; ++v)
                    for (int p = 0; p < nf; ++p) {
                        size_t o = (size_t)p + nf * (i + (size_t)fx * (j + (size_t)fy * (k + (size_t)fz * v)));
                        flux[o] = 0.5 * (ff[v * nfe + p] + ff[v * nfe + p + nf]) -
                                  0.5 * cfr[p] * (Qf[v * nfe + p + nf] - Qf[v * nfe + p]);
                    }
                if (c->p.ihllc == 1) {
                    flux_hllc(c, Qf, ff, fh, d);
                    for (int v = 0; v < 5; ++v)
                        for (int p = 0; p < nf; ++p) {
                            size_t o = (size_t)p + nf * (i + (size_t)fx * (j + (size_t)fy * (k + (size_t)fz * v)));
                            flux[o] = fh[v * nf + p];
                        }
                } else if (c->p.ihllc == 2) {
                    int kroe[16];
                    flux_roe(c, Qf, ff, fh, kroe, d);
                    for (int v = 0; v < 5; ++v)
                        for (int p = 0; p < nf; ++p)
                            if (kroe[p] > 0) {
                                size_t o = (size_t)p + nf * (i + (size_t)fx * (j + (size_t)fy * (k + (size_t)fz * v)));
                                flux[o] = fh[v * nf + p];
                            }
                }
            }
        }
}

/* flux.f90:751-928 innerintegral2 */
static void innerintegral2(orc_ctx *c, const double *Q) {
    const int nx = c->nx, ny = c->ny, nz = c->nz, npg = c->npg, nb = c->nb;
    const double dxi = c->dxi, dyi = c->dyi, dzi = c->dzi;
    const double *cb = c->cbasis, *w = c->wgt3d + 1, *bi = c->bfvals_int;
    const int ib = c->ibitri, iq = c->iquad;
    const int noise = c->p.llns ? NOISE_INT_X : -1;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j) {
            double Qin[64 * NQ], fx_[64 * NQ], fy_[64 * NQ], fz_[64 * NQ], ir_[(NBT + 1) * NQ];
            for (int i = 0; i < nx; ++i) {
                for (int v = 0; v < NQ; ++v)
                    for (int g = 0; g < npg; ++g) Qin[v * npg + g] = trace(c, bi, g, Q, i, j, k, v);
                unsigned long long site = (unsigned long long)i + (unsigned long long)nx * (j + (unsigned long long)ny * k);
                flux_calc_pnts_r(c, Qin, fx_, 1, npg, noise < 0 ? -1 : NOISE_INT_X, site);
                flux_calc_pnts_r(c, Qin, fy_, 2, npg, noise < 0 ? -1 : NOISE_INT_Y, site);
                flux_calc_pnts_r(c, Qin, fz_, 3, npg, noise < 0 ? -1 : NOISE_INT_Z, site);
                for (int b = 0; b <= NBT; ++b)
                    for (int v = 0; v < NQ; ++v) ir_[b * NQ + v] = 0.;
#define FX(g) fx_[v * npg + (g)]
#define FY(g) fy_[v * npg + (g)]
#define FZ(g) fz_[v * npg + (g)]
#define BV(g, b) TB(bi, g, b)
#define IR(b) ir_[(b) * NQ + v]
                for (int v = 0; v < NQ; ++v) {
                    double s1 = 0., s2 = 0., s3 = 0.;
                    for (int g = 0; g < npg; ++g) {
                        s1 = s1 + w[g] * FX(g);
                        s2 = s2 + w[g] * FY(g);
                        s3 = s3 + w[g] * FZ(g);
                    }
                    IR(c->kx) = 0.25 * cb[c->kx] * dxi * s1;
                    IR(c->ky) = 0.25 * cb[c->ky] * dyi * s2;
                    IR(c->kz) = 0.25 * cb[c->kz] * dzi * s3;
                    if (nb > 4) {
                        if (ib == 1 || iq > 2) {
                            double a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0, a6 = 0;
                            for (int g = 0; g < npg; ++g) {
                                a1 = a1 + w[g] * BV(g, c->kz) * FY(g);
                                a2 = a2 + w[g] * BV(g, c->ky) * FZ(g);
                                a3 = a3 + w[g] * BV(g, c->kz) * FX(g);
                                a4 = a4 + w[g] * BV(g, c->kx) * FZ(g);
                                a5 = a5 + w[g] * BV(g, c->ky) * FX(g);
                                a6 = a6 + w[g] * BV(g, c->kx) * FY(g);
                            }
                            IR(c->kyz) = 0.25 * cb[c->kyz] * (dyi * a1 + dzi * a2);
                            IR(c->kzx) = 0.25 * cb[c->kzx] * (dxi * a3 + dzi * a4);
                            IR(c->kxy) = 0.25 * cb[c->kxy] * (dxi * a5 + dyi * a6);
                        }
                        if (iq > 2) {
                            double a1 = 0, a2 = 0, a3 = 0;
                            for (int g = 0; g < npg; ++g) {
                                a1 = a1 + w[g] * 3. * BV(g, c->kx) * FX(g);
                                a2 = a2 + w[g] * 3. * BV(g, c->ky) * FY(g);
                                a3 = a3 + w[g] * 3. * BV(g, c->kz) * FZ(g);
                            }
                            IR(c->kxx) = 0.25 * cb[c->kxx] * (dxi * a1);
                            IR(c->kyy) = 0.25 * cb[c->kyy] * (dyi * a2);
                            IR(c->kzz) = 0.25 * cb[c->kzz] * (dzi * a3);
                        }
                        if (ib == 1 || iq > 3) {
                            double a7 = 0, a8 = 0, a9 = 0;
                            for (int g = 0; g < npg; ++g) {
                                a7 = a7 + w[g] * BV(g, c->kyz) * FX(g);
                                a8 = a8 + w[g] * BV(g, c->kzx) * FY(g);
                                a9 = a9 + w[g] * BV(g, c->kxy) * FZ(g);
                            }
                            IR(c->kxyz) = 0.25 * cb[c->kxyz] * (dxi * a7 + dyi * a8 + dzi * a9);
                        }
                        /* the remaining families: sum(w * dphi * F) per direction */
#define S1(bb, F) ({ double _s = 0.; for (int g = 0; g < npg; ++g) _s += w[g] * BV(g, bb) * F(g); _s; })
#define S3(bb, F) ({ double _s = 0.; for (int g = 0; g < npg; ++g) _s += w[g] * 3. * BV(g, bb) * F(g); _s; })
                        if ((ib == 1 && iq > 2) || iq > 3) {
                            IR(c->kyzz) = 0.25 * cb[c->kyzz] * dyi * S1(c->kzz, FY) + 0.25 * cb[c->kyzz] * dzi * S3(c->kyz, FZ);
                            IR(c->kzxx) = 0.25 * cb[c->kzxx] * dzi * S1(c->kxx, FZ) + 0.25 * cb[c->kzxx] * dxi * S3(c->kzx, FX);
                            IR(c->kxyy) = 0.25 * cb[c->kxyy] * dxi * S1(c->kyy, FX) + 0.25 * cb[c->kxyy] * dyi * S3(c->kxy, FY);
                            IR(c->kyyz) = 0.25 * cb[c->kyyz] * dzi * S1(c->kyy, FZ) + 0.25 * cb[c->kyyz] * dyi * S3(c->kyz, FY);
                            IR(c->kzzx) = 0.25 * cb[c->kzzx] * dxi * S1(c->kzz, FX) + 0.25 * cb[c->kzzx] * dzi * S3(c->kzx, FZ);
                            IR(c->kxxy) = 0.25 * cb[c->kxxy] * dyi * S1(c->kxx, FY) + 0.25 * cb[c->kxxy] * dxi * S3(c->kxy, FX);
                        }
                        if (iq > 3) {
                            double a1 = 0, a2 = 0, a3 = 0;
                            for (int g = 0; g < npg; ++g) {
                                a1 += w[g] * (7.5 * BV(g, c->kx) * BV(g, c->kx) - 1.5) * FX(g);
                                a2 += w[g] * (7.5 * BV(g, c->ky) * BV(g, c->ky) - 1.5) * FY(g);
                                a3 += w[g] * (7.5 * BV(g, c->kz) * BV(g, c->kz) - 1.5) * FZ(g);
                            }
                            IR(c->kxxx) = 0.25 * cb[c->kxxx] * dxi * a1;
                            IR(c->kyyy) = 0.25 * cb[c->kyyy] * dyi * a2;
                            IR(c->kzzz) = 0.25 * cb[c->kzzz] * dzi * a3;
                        }
                        if (ib == 1 && iq > 2) {
                            IR(c->kyyzz) = 0.25 * cb[c->kyyzz] * dyi * S3(c->kyzz, FY) + 0.25 * cb[c->kyyzz] * dzi * S3(c->kyyz, FZ);
                            IR(c->kzzxx) = 0.25 * cb[c->kzzxx] * dzi * S3(c->kzxx, FZ) + 0.25 * cb[c->kzzxx] * dxi * S3(c->kzzx, FX);
                            IR(c->kxxyy) = 0.25 * cb[c->kxxyy] * dxi * S3(c->kxyy, FX) + 0.25 * cb[c->kxxyy] * dyi * S3(c->kxxy, FY);
                            IR(c->kyzxx) = 0.25 * cb[c->kyzxx] * dxi * S3(c->kxyz, FX) + 0.25 * cb[c->kyzxx] * dyi * S1(c->kzxx, FY) +
                                           0.25 * cb[c->kyzxx] * dzi * S1(c->kxxy, FZ);
                            IR(c->kzxyy) = 0.25 * cb[c->kzxyy] * dyi * S3(c->kxyz, FY) + 0.25 * cb[c->kzxyy] * dzi * S1(c->kxyy, FZ) +
                                           0.25 * cb[c->kzxyy] * dxi * S1(c->kyyz, FX);
                            IR(c->kxyzz) = 0.25 * cb[c->kxyzz] * dzi * S3(c->kxyz, FZ) + 0.25 * cb[c->kxyzz] * dxi * S1(c->kyzz, FX) +
                                           0.25 * cb[c->kxyzz] * dyi * S1(c->kzzx, FY);
                            IR(c->kxyyzz) = 0.25 * cb[c->kxyyzz] * dxi * S1(c->kyyzz, FX) + 0.25 * cb[c->kxyyzz] * dyi * S3(c->kxyzz, FY) +
                                            0.25 * cb[c->kxyyzz] * dzi * S3(c->kzxyy, FZ);
                            IR(c->kyzzxx) = 0.25 * cb[c->kyzzxx] * dyi * S1(c->kzzxx, FY) + 0.25 * cb[c->kyzzxx] * dzi * S3(c->kyzxx, FZ) +
                                            0.25 * cb[c->kyzzxx] * dxi * S3(c->kxyzz, FX);
                            IR(c->kzxxyy) = 0.25 * cb[c->kzxxyy] * dzi * S1(c->kxxyy, FZ) + 0.25 * cb[c->kzxxyy] * dxi * S3(c->kzxyy, FX) +
                                            0.25 * cb[c->kzxxyy] * dyi * S3(c->kyzxx, FY);
                            IR(c->kxxyyzz) = 0.25 * cb[c->kxxyyzz] * dxi * S3(c->kxyyzz, FX) + 0.25 * cb[c->kxxyyzz] * dyi * S3(c->kyzzxx, FY) +
                                             0.25 * cb[c->kxxyyzz] * dzi * S3(c->kzxxyy, FZ);
                        }
#undef S1
#undef S3
                    }
                }
#undef FX
#undef FY
#undef FZ
#undef BV
#undef IR
                for (int v = 0; v < NQ; ++v)
                    for (int b = 1; b <= nb; ++b) c->integral_r[QI(c, i, j, k, v, b - 1)] = ir_[b * NQ + v];
            }
        }
}

/* flux.f90:932-1022 glflux: surface assembly minus the volume integral */
static void glflux_assemble(orc_ctx *c) {
    const int nx = c->nx, ny = c->ny, nz = c->nz, nf = c->nface, nb = c->nb;
    const double *w2 = c->wgt2d + 1, *cb = c->cbasis;
    for (int v = 0; v < NQ; ++v)
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
#define FXI(p, ii) c->flux_x[(size_t)(p) + nf * ((ii) + (size_t)(nx + 1) * (j + (size_t)ny * (k + (size_t)nz * v)))]
#define FYI(p, jj) c->flux_y[(size_t)(p) + nf * (i + (size_t)nx * ((jj) + (size_t)(ny + 1) * (k + (size_t)nz * v)))]
#define FZI(p, kk) c->flux_z[(size_t)(p) + nf * (i + (size_t)nx * (j + (size_t)ny * ((kk) + (size_t)(nz + 1) * v)))]
                    double sx = 0., sy = 0., sz = 0.;
                    for (int p = 0; p < nf; ++p) sx = sx + w2[p] * (FXI(p, i + 1) - FXI(p, i));
                    for (int p = 0; p < nf; ++p) sy = sy + w2[p] * (FYI(p, j + 1) - FYI(p, j));
                    for (int p = 0; p < nf; ++p) sz = sz + w2[p] * (FZI(p, k + 1) - FZI(p, k));
                    c->glflux_r[QI(c, i, j, k, v, 0)] = 0.25 * (c->dxi * sx + c->dyi * sy + c->dzi * sz);
                    for (int b = 2; b <= nb; ++b) {
                        sx = 0.; sy = 0.; sz = 0.;
                        for (int p = 0; p < nf; ++p)
                            sx = sx + w2[p] * (TB(c->bfvals_xp, p, b) * FXI(p, i + 1) - TB(c->bfvals_xm, p, b) * FXI(p, i));
                        for (int p = 0; p < nf; ++p)
                            sy = sy + w2[p] * (TB(c->bfvals_yp, p, b) * FYI(p, j + 1) - TB(c->bfvals_ym, p, b) * FYI(p, j));
                        for (int p = 0; p < nf; ++p)
                            sz = sz + w2[p] * (TB(c->bfvals_zp, p, b) * FZI(p, k + 1) - TB(c->bfvals_zm, p, b) * FZI(p, k));
                        c->glflux_r[QI(c, i, j, k, v, b - 1)] =
                            0.25 * cb[b] * (c->dxi * sx + c->dyi * sy + c->dzi * sz) - c->integral_r[QI(c, i, j, k, v, b - 1)];
                    }
#undef FXI
#undef FYI
#undef FZI
                }
}

/* sources.f90:12-84 source_calc */
static void source_calc(orc_ctx *c, const double *Q) {
    const int nx = c->nx, ny = c->ny, nz = c->nz, npg = c->npg, nb = c->nb;
    size_t n = (size_t)nx * ny * nz * NQ * nb;
    if ((c->p.ivis == 1 || c->p.ivis == 3) && c->p.body_force == 0.0) {  /* every point source is 0 in this mode */
        memset(c->source_r, 0, n * sizeof(double));
        return;
    }
    const double gforce = c->p.body_force;
    const double coll = c->p.coll;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j) {
            double src[64 * NQ];
            for (int i = 0; i < nx; ++i) {
                for (int g = 0; g < npg; ++g) {
                    double Qin[NQ];
                    for (int v = 0; v < NQ; ++v) Qin[v] = trace(c, c->bfvals_int, g, Q, i, j, k, v);
                    for (int v = RH; v <= EN; ++v) src[v * npg + g] = 0;
                    /* body force (new term): d(mx)/dt += rho g, d(en)/dt += mx g */
                    if (gforce != 0.0) {
                        src[MX * npg + g] = Qin[RH] * gforce;
                        src[EN * npg + g] = Qin[MX] * gforce;
                    }
                    if (c->p.ivis == 1 || c->p.ivis == 3) {
                        for (int v = PXX; v <= PYZ; ++v) src[v * npg + g] = 0;
                    } else if (c->p.ivis == 0) {
                        for (int v = PXX; v <= PYZ; ++v) src[v * npg + g] = -coll * Qin[v];
                    } else {
                        double dn = Qin[RH], dni = 1. / dn;
                        double vx = Qin[MX] * dni, vy = Qin[MY] * dni, vz = Qin[MZ] * dni;
                        double vx2 = vx * vx, vy2 = vy * vy, vz2 = vz * vz;
                        double colldn = coll * dn;
                        src[PXX * npg + g] = colldn * (2 * vx2 - vy2 - vz2) * c->c1d3;
                        src[PYY * npg + g] = colldn * (2 * vy2 - vz2 - vx2) * c->c1d3;
                        src[PZZ * npg + g] = colldn * (2 * vz2 - vx2 - vy2) * c->c1d3;
                        src[PXY * npg + g] = colldn * vx * vy;
                        src[PXZ * npg + g] = colldn * vx * vz;
                        src[PYZ * npg + g] = colldn * vy * vz;
                    }
                }
                for (int b = 1; b <= nb; ++b)
                    for (int v = 0; v < NQ; ++v) {
                        double s = 0.;
                        for (int g = 0; g < npg; ++g) s += TB(c->bval_int_wgt, g, b) * src[v * npg + g];
                        c->source_r[QI(c, i, j, k, v, b - 1)] = 0.125 * c->cbasis[b] * s;
                    }
            }
        }
}

/* flux.f90:1077-1164 limiter, in place */
void orc_limiter(orc_ctx *c, double *Q) {
    const int nx = c->nx, ny = c->ny, nz = c->nz, nb = c->nb, npge = c->npge;
    const double epsi = c->p.rh_floor, epsiP = c->p.rh_floor * c->p.T_floor;
    const double aindm1 = c->aindm1;
    double t0 = wtime();
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
#define QQ(v, b) Q[QI(c, i, j, k, v, b)]
                if (QQ(RH, 0) < c->p.rh_floor) {
                    for (int b = 1; b < nb; ++b)
                        for (int v = RH; v <= EN; ++v) QQ(v, b) = 0.0;
                    QQ(RH, 0) = c->p.rh_floor;
                } else {
                    double Qrhmin = INFINITY;
                    for (int pg = 0; pg < npge; ++pg) {
                        double s = 0.;
                        for (int b = 1; b <= nb; ++b) s += TB(c->bf_faces, pg, b) * QQ(RH, b - 1);
                        if (pg == 0 || s < Qrhmin) Qrhmin = s;
                    }
                    if (Qrhmin < epsi) {
                        double theta = (epsi - QQ(RH, 0)) / (Qrhmin - QQ(RH, 0));
                        if (theta > 1.) theta = 1.;
                        if (theta < 0) theta = 0.;
                        for (int b = 1; b < nb; ++b) QQ(RH, b) = fabs(theta) * QQ(RH, b);
                    }
                    double Pave = aindm1 * (QQ(EN, 0) - 0.5 * (QQ(MX, 0) * QQ(MX, 0) + QQ(MY, 0) * QQ(MY, 0) + QQ(MZ, 0) * QQ(MZ, 0)) / QQ(RH, 0));
                    if (Pave < epsiP) {
                        for (int b = 1; b < nb; ++b)
                            for (int v = RH; v <= EN; ++v) QQ(v, b) = 0.0;
                    } else {
                        double theta = 1.;
                        for (int pg = 0; pg < npge; ++pg) {
                            double qe[5];
                            for (int v = RH; v <= EN; ++v) {
                                double s = 0.;
                                for (int b = 1; b <= nb; ++b) s += TB(c->bf_faces, pg, b) * QQ(v, b - 1);
                                qe[v] = s;
                            }
                            double dn = qe[RH], dni = 1. / dn;
                            double P = aindm1 * (qe[EN] - 0.5 * dni * (qe[MX] * qe[MX] + qe[MY] * qe[MY] + qe[MZ] * qe[MZ]));
                            if (P < epsiP) {
                                if (Pave != P) {
                                    double thetaj = (Pave - epsiP) / (Pave - P);
                                    theta = fmin(theta, thetaj);
                                }
                            }
                        }
                        if (theta > 1.) theta = 1.;
                        if (theta < 0.) theta = 0.;
                        for (int b = 1; b < nb; ++b)
                            for (int v = RH; v <= EN; ++v) QQ(v, b) = theta * QQ(v, b);
                    }
                }
#undef QQ
            }
    c->timers[0] += wtime() - t0;
}

static void calc_rhs(orc_ctx *c, const double *Q) {
    double t0 = wtime();
    exchange_and_bc(c, Q);
    calc_flux_dir(c, Q, 1);
    calc_flux_dir(c, Q, 2);
    calc_flux_dir(c, Q, 3);
    double t1 = wtime();
    innerintegral2(c, Q);
    double t2 = wtime();
    glflux_assemble(c);
    double t3 = wtime();
    source_calc(c, Q);
    double t4 = wtime();
    c->timers[1] += t1 - t0; c->timers[2] += t2 - t1; c->timers[3] += t3 - t2; c->timers[4] += t4 - t3;
}

void orc_rhs_nolimit(orc_ctx *c, const double *Q, double *rhs) {
    calc_rhs(c, Q);
    size_t n = (size_t)orc_qsize(c);
    for (size_t e = 0; e < n; ++e) rhs[e] = c->glflux_r[e] - c->source_r[e];
}

void orc_prep_and_rhs(orc_ctx *c, double *Q, double *rhs) {
    if (c->p.ieos == 1 || c->p.ieos == 2) orc_limiter(c, Q);
    orc_rhs_nolimit(c, Q, rhs);
}

/* integrator.f90:125-252 advance_time_level */
static void advance_time_level(orc_ctx *c, const double *Qin, double *Qout, double dt) {
    const int nb = c->nb;
    const size_t nc = (size_t)c->nx * c->ny * c->nz;
    const double coll = c->p.coll, c1d3 = c->c1d3;
    const double faci = 1. / (1. + dt * coll);
    const double *gl = c->glflux_r, *sr = c->source_r;
    double t0 = wtime();
#define IX(v, b, e) ((e) + nc * ((v) + (size_t)NQ * (b)))
    if (c->p.ivis == 0 || c->p.ivis == 3) {
        /* ivis 3: advance_time_level_gl (ten_moment.f90:795-837) with fac = 1 */
#pragma omp parallel for
        for (long e = 0; e < (long)(nc * NQ * nb); ++e) Qout[e] = Qin[e] - dt * (gl[e] - sr[e]);
    } else if (c->p.ivis == 1) {
#pragma omp parallel for
        for (long e = 0; e < (long)(nc * NQ * nb); ++e) {
            long v = (e / (long)nc) % NQ;
            double q = Qin[e] - dt * (gl[e] - sr[e]);
            Qout[e] = (v >= PXX) ? faci * q : q;
        }
    } else {
#pragma omp parallel for
        for (long e = 0; e < (long)(nc * NQ * nb); ++e) {
            long v = (e / (long)nc) % NQ;
            /* integrator.f90:181-228 leaves rh..en of Q_out unwritten (ivis 2
             * is marked unfinished there); they get the explicit update of
             * the ivis-0 branch here, as in the CUDA path */
            if (v <= EN) Qout[e] = Qin[e] - dt * (gl[e] - sr[e]);
        }
#pragma omp parallel for
        for (long ee = 0; ee < (long)(nc * nb); ++ee) {
            size_t e = (size_t)ee % nc, b = (size_t)ee / nc;
            double P_xx = Qin[IX(PXX, b, e)], P_yy = Qin[IX(PYY, b, e)], P_zz = Qin[IX(PZZ, b, e)];
            double g_xx = gl[IX(PXX, b, e)], g_yy = gl[IX(PYY, b, e)], g_zz = gl[IX(PZZ, b, e)];
            double s_xx = sr[IX(PXX, b, e)], s_yy = sr[IX(PYY, b, e)], s_zz = sr[IX(PZZ, b, e)];
            double Q_sum = coll * dt * (P_xx + P_yy + P_zz) * c1d3;
            double glf_sum = coll * (dt * dt) * (g_xx + g_yy + g_zz) * c1d3;
            double src_sum = coll * (dt * dt) * (s_xx + s_yy + s_zz) * c1d3;
            Qout[IX(PXX, b, e)] = faci * (P_xx - dt * g_xx + dt * s_xx + Q_sum - glf_sum + src_sum);
            Qout[IX(PYY, b, e)] = faci * (P_yy - dt * g_yy + dt * s_yy + Q_sum - glf_sum + src_sum);
            Qout[IX(PZZ, b, e)] = faci * (P_zz - dt * g_zz + dt * s_zz + Q_sum - glf_sum + src_sum);
            for (int v = PXY; v < NQ; ++v) Qout[IX(v, b, e)] = (Qin[IX(v, b, e)] - dt * gl[IX(v, b, e)] + dt * sr[IX(v, b, e)]) * faci;
        }
    }
    /* integrator.f90:234-250: NaN on a cell average (the reference exits) */
    for (int v = 0; v < NQ; ++v)
        for (size_t e = 0; e < nc; ++e)
            if (Qout[IX(v, 0, e)] != Qout[IX(v, 0, e)]) c->nonfinite = 1;
#undef IX
    c->timers[5] += wtime() - t0;
}

/* Grad closure (ivis 3), the operator-split implicit relaxation step of
 * dg_3D_hydro_bitri_ten_moment.f90:719-793 (source_calc) and :839-892
 * (advance_time_level_source), in place on Q.  The reference calls it with
 * the same array as input and output (non-conforming aliasing whose result
 * depends on the compiler); here every update reads the values before the
 * step. */
static void source_split(orc_ctx *c, double *Q, double dt) {
    const int nx = c->nx, ny = c->ny, nz = c->nz, npg = c->npg, nb = c->nb;
    const double coll = c->p.coll, oth = 1. / 3.;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double S[6][64];
                for (int g = 0; g < npg; ++g) {
                    double dn = trace(c, c->bfvals_int, g, Q, i, j, k, RH), dni = 1. / dn;
                    double vx = trace(c, c->bfvals_int, g, Q, i, j, k, MX) * dni;
                    double vy = trace(c, c->bfvals_int, g, Q, i, j, k, MY) * dni;
                    double vz = trace(c, c->bfvals_int, g, Q, i, j, k, MZ) * dni;
                    double cd = coll * dn;
                    S[0][g] = cd * (2 * vx * vx - vy * vy - vz * vz) * oth;
                    S[1][g] = cd * (2 * vy * vy - vz * vz - vx * vx) * oth;
                    S[2][g] = cd * (2 * vz * vz - vx * vx - vy * vy) * oth;
                    S[3][g] = cd * vx * vy;
                    S[4][g] = cd * vx * vz;
                    S[5][g] = cd * vy * vz;
                }
                for (int b = 1; b <= nb; ++b) {
                    double sr[6], E[6];
                    for (int m = 0; m < 6; ++m) {
                        double s = 0.;
                        for (int g = 0; g < npg; ++g) s += TB(c->bval_int_wgt, g, b) * S[m][g];
                        sr[m] = 0.125 * c->cbasis[b] * s;
                        E[m] = Q[QI(c, i, j, k, PXX + m, b - 1)];
                    }
                    double den = 1. + dt * coll;
                    double Esum = coll * dt * (E[0] + E[1] + E[2]) * oth;
                    double Ssum = coll * (dt * dt) * (sr[0] + sr[1] + sr[2]) * oth;
                    for (int m = 0; m < 3; ++m) Q[QI(c, i, j, k, PXX + m, b - 1)] = (E[m] + dt * sr[m] + Esum + Ssum) / den;
                    for (int m = 3; m < 6; ++m) Q[QI(c, i, j, k, PXX + m, b - 1)] = (E[m] + dt * sr[m]) / den;
                }
            }
}

/* integrator.f90:93-122 euler_step */
void orc_euler_step(orc_ctx *c, double *Qin, double *Qout, double dt) {
    if (c->p.ieos == 1 || c->p.ieos == 2) orc_limiter(c, Qin);
    calc_rhs(c, Qin);
    advance_time_level(c, Qin, Qout, dt);
    /* ten_moment.f90:342-361: RK2 follows each advection stage by the source step */
    if (c->p.ivis == 3 && c->p.iorder == 2) source_split(c, Qout, dt);
    c->noise_stage++;
}

/* hermeshd.f90:145-199 get_min_dt (single rank: the min-reduce is the identity) */
double orc_get_min_dt(orc_ctx *c, const double *Q) {
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    double vmag = 0., cs = 0.;
    const double aindex = c->p.aindex;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double dn = Q[QI(c, i, j, k, RH, 0)], dni = 1. / dn;
                double vx = Q[QI(c, i, j, k, MX, 0)] * dni, vy = Q[QI(c, i, j, k, MY, 0)] * dni, vz = Q[QI(c, i, j, k, MZ, 0)] * dni;
                if (c->p.ieos == 1) cs = sqrt(aindex * (Q[QI(c, i, j, k, EN, 0)] * dni - 0.5 * (vx * vx + vy * vy + vz * vz)));
                if (c->p.ieos == 2) cs = sqrt(7.2 * c->p.P_1 * pow(dn, 6.2) + c->p.T_floor);
                double vmag0 = fmax(fmax(fabs(vx) + cs, fabs(vy) + cs), fabs(vz) + cs);
                if (vmag0 > vmag && dn > c->p.rh_mult * c->p.rh_floor) vmag = vmag0;
            }
    /* hermeshd.f90:174: the sound speed of the last cell, and dxi only */
    double vmax = (vmag + cs) * c->dxi;
    return c->cflm / vmax;
}

/* integrator.f90:62-86 RK2 / RK3 */
static void rk_update(orc_ctx *c, double *Q, double *Q1, double *Q2, double dt) {
    size_t n = (size_t)orc_qsize(c);
    c->noise_stage = 0;
    if (c->p.iorder == 3) {
        orc_euler_step(c, Q, Q1, dt);
        orc_euler_step(c, Q1, Q2, dt);
        for (size_t e = 0; e < n; ++e) Q1[e] = 0.75 * Q[e] + 0.25 * Q2[e];
        orc_euler_step(c, Q1, Q2, dt);
        for (size_t e = 0; e < n; ++e) Q[e] = c->c1d3 * Q[e] + c->c2d3 * Q2[e];
    } else {
        orc_euler_step(c, Q, Q1, dt);
        orc_euler_step(c, Q1, Q2, dt);
        for (size_t e = 0; e < n; ++e) Q[e] = 0.5 * (Q[e] + Q2[e]);
    }
    c->noise_step++;
}

void orc_step(orc_ctx *c, double *Q, double *Q1, double *Q2, double *t, double *dt) {
    *dt = orc_get_min_dt(c, Q);
    rk_update(c, Q, Q1, Q2, *dt);
    *t = *t + *dt;
}

int orc_advance(orc_ctx *c, double *Q, double *Q1, double *Q2, double *t, double *dt, int nsteps) {
    c->nonfinite = 0;
    for (int s = 0; s < nsteps; ++s) {
        orc_step(c, Q, Q1, Q2, t, dt);
        if (c->nonfinite) return -(s + 1);
    }
    return nsteps;
}

void orc_advance_fixed_dt(orc_ctx *c, double *Q, double *Q1, double *Q2, double dt, int nsteps) {
    for (int s = 0; s < nsteps; ++s) rk_update(c, Q, Q1, Q2, dt);
}

void orc_set_noise_counter(orc_ctx *c, unsigned long long step) { c->noise_step = step; c->noise_stage = 0; }

void orc_get_timers(const orc_ctx *c, double *o) { for (int i = 0; i < 6; ++i) o[i] = c->timers[i]; }
void orc_reset_timers(orc_ctx *c) { for (int i = 0; i < 6; ++i) c->timers[i] = 0; }
int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* basis_funcs.f90:634-992 test_basis_3D: cell scalar products
 * 0.125*cbasis(i)*sum(w3*phi_i*phi_j) must be the identity.  The face part
 * checks the x/y/z face scalar products against the reference's expected
 * pattern, which for the families here reduces to: the product over a face
 * of two basis functions with equal tangential parts is (face norm)^2, else 0.
 * Returned: max deviation of the cell products, and of the face products
 * recomputed as 0.25*sum(w2*phi_i*phi_j)*c_i*c_j against delta over the
 * tangential family. */
double orc_test_basis(const orc_ctx *c, double *cell_dev, double *face_dev) {
    int nb = c->nb;
    double md = 0.;
    for (int jr = 1; jr <= nb; ++jr)
        for (int ir = 1; ir <= nb; ++ir) {
            double s = 0.;
            for (int g = 0; g < c->npg; ++g) s += c->wgt3d[g + 1] * TB(c->bfvals_int, g, ir) * TB(c->bfvals_int, g, jr);
            double ci = 0.125 * c->cbasis[ir] * s;
            double d = fabs(ci - (ir == jr ? 1. : 0.));
            if (d > md) md = d;
        }
    if (cell_dev) *cell_dev = md;
    /* face products: Gram matrix of the traces on each face, normalised by
     * its own diagonal; identical traces (a function and its product with the
     * normal coordinate) give 1, distinct tangential families give 0 */
    double mf = 0.;
    const double *tabs[6] = {c->bfvals_xm, c->bfvals_xp, c->bfvals_ym, c->bfvals_yp, c->bfvals_zm, c->bfvals_zp};
    for (int f = 0; f < 6; ++f)
        for (int jr = 1; jr <= nb; ++jr)
            for (int ir = 1; ir <= nb; ++ir) {
                double sij = 0., sii = 0., sjj = 0.;
                for (int p = 0; p < c->nface; ++p) {
                    double a = TB(tabs[f], p, ir), b = TB(tabs[f], p, jr);
                    sij += c->wgt2d[p + 1] * a * b;
                    sii += c->wgt2d[p + 1] * a * a;
                    sjj += c->wgt2d[p + 1] * b * b;
                }
                double cosang = sij / sqrt(sii * sjj);
                double d = fmin(fabs(cosang), fabs(fabs(cosang) - 1.));
                if (d > mf) mf = d;
            }
    if (face_dev) *face_dev = mf;
    return md > mf ? md : mf;
}

void orc_noise_sample(unsigned long long seed, unsigned long long step, unsigned stage, unsigned kind,
                      unsigned long long site, unsigned pt, double eta, double zeta, double G6[6], double S6[6]) {
    orc_ctx c;
    memset(&c, 0, sizeof(c));
    c.p.seed = seed;
    c.p.eta_sd = eta;
    c.p.zeta_sd = zeta;
    c.noise_step = step;
    c.noise_stage = (int)stage;
    hermes_philox_normals6(seed, step, stage, kind, site, pt, G6);
    stress_at(&c, (int)kind, site, (int)pt, S6);
}

/* one Philox-4x32-10 block, for known-answer tests of the generator */
void orc_philox4x32_10(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
    hermes_philox4x32_10(ctr, k0, k1, out);
}

/*
 * philox_ref.h -- Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
 * random numbers: as easy as 1, 2, 3", SC'11) and a Box-Muller transform,
 * restated in plain C for the oracle.  TEST INFRASTRUCTURE ONLY.
 *
 * The reference draws its stochastic-stress normals from Intel MKL VSL
 * (MCG31 + Box-Muller, random.f90:17-18,61), which is not vendored and not
 * reproducible here; the stress path is disabled in the reference
 * (flux.f90:41).  This file fixes the counter scheme shared with the CUDA
 * kernels so that a run with noise on is reproducible:
 *   key     = seed (64 bit)
 *   counter = (site, pt | kind<<8 | sub<<12 | stage<<16, step_lo, step_hi)
 * where site is the face or cell index, pt the quadrature point of the call,
 * kind the flux call (face x/y/z, interior x/y/z), sub the Philox block
 * (0, 1) and stage the RK stage.  The stress needs six independent normals
 * per point (random.f90 symmetrises a 3x3 matrix of nine: its three diagonal
 * entries and the three scaled sums sqrt(1/2) (G_ij + G_ji) are six
 * independent N(0,1) values, drawn here directly).  Each 32-bit output word
 * is one uniform in (0,1), (w + 1/2) 2^-32; two blocks give eight, and three
 * Box-Muller pairs of the first six give the six normals.
 */
#ifndef HERMES_PHILOX_REF_H
#define HERMES_PHILOX_REF_H

#include <math.h>
#include <stdint.h>

static inline void hermes_philox4x32_10(const uint32_t ctr_in[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* uniform in (0,1) from one 32-bit word */
static inline double hermes_u32(uint32_t w) { return ((double)w + 0.5) * (1.0 / 4294967296.0); }

/* six N(0,1) values for one quadrature point of one flux call: the diagonal
 * (xx, yy, zz) and off-diagonal (xy, xz, yz) normals of the stress */
static inline void hermes_philox_normals6(unsigned long long seed, unsigned long long step, unsigned stage,
                                          unsigned kind, unsigned long long site, unsigned pt, double G[6]) {
    const double two_pi = 6.283185307179586476925286766559;
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    uint32_t w[8];
    for (unsigned sub = 0; sub < 2; ++sub) {
        uint32_t ctr[4];
        ctr[0] = (uint32_t)site;
        ctr[1] = (pt & 0xFFu) | ((kind & 0xFu) << 8) | ((sub & 0xFu) << 12) | ((stage & 0xFFFFu) << 16);
        ctr[2] = (uint32_t)step;
        ctr[3] = (uint32_t)(step >> 32);
        hermes_philox4x32_10(ctr, k0, k1, w + 4 * sub);
    }
    for (int k = 0; k < 3; ++k) {
        double u1 = hermes_u32(w[2 * k]), u2 = hermes_u32(w[2 * k + 1]);
        double r = sqrt(-2.0 * log(u1));
        G[2 * k] = r * cos(two_pi * u2);
        G[2 * k + 1] = r * sin(two_pi * u2);
    }
}

#endif

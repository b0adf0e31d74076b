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
 * (0..4) and stage the RK stage.  Each block gives two 53-bit uniforms and
 * one Box-Muller pair; nine normals per point use five blocks.
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

/* 53-bit uniform in (0,1) from two 32-bit words */
static inline double hermes_u53(uint32_t a, uint32_t b) {
    uint64_t m = ((uint64_t)a << 21) | (uint64_t)(b >> 11);
    return ((double)m + 0.5) * (1.0 / 9007199254740992.0);
}

/* nine N(0,1) values for one quadrature point of one flux call */
static inline void hermes_philox_normals9(unsigned long long seed, unsigned long long step, unsigned stage,
                                          unsigned kind, unsigned long long site, unsigned pt, double G[9]) {
    const double two_pi = 6.283185307179586476925286766559;
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    double z[10];
    for (unsigned sub = 0; sub < 5; ++sub) {
        uint32_t ctr[4], o[4];
        ctr[0] = (uint32_t)site;
        ctr[1] = (pt & 0xFFu) | ((kind & 0xFu) << 8) | ((sub & 0xFu) << 12) | ((stage & 0xFFFFu) << 16);
        ctr[2] = (uint32_t)step;
        ctr[3] = (uint32_t)(step >> 32);
        hermes_philox4x32_10(ctr, k0, k1, o);
        double u1 = hermes_u53(o[0], o[1]), u2 = hermes_u53(o[2], o[3]);
        double r = sqrt(-2.0 * log(u1));
        z[2 * sub] = r * cos(two_pi * u2);
        z[2 * sub + 1] = r * sin(two_pi * u2);
    }
    for (int i = 0; i < 9; ++i) G[i] = z[i];
}

#endif

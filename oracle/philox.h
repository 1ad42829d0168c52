/*
 * Oracle copy of the sampler's random-number schedule -- TEST INFRASTRUCTURE.
 *
 * Philox-4x32-10 (Salmon et al., "Parallel random numbers: as easy as
 * 1, 2, 3", SC'11), written from the published round function:
 *   (L0,R0,L1,R1) -> (hi(M1*R1)^L0^k0 ... ) with multipliers 0xD2511F53,
 *   0xCD9E8D57 and Weyl key increments 0x9E3779B9, 0xBB67AE85.
 *
 * Schedule (the contract the device sampler follows as well):
 *   key     = {seed, chain_id}
 *   counter = {lo32(n), hi32(n), stream, 0}, n = per-stream draw index
 *   stream 0: sampler draws (jitter, momentum, direction, multinomial)
 *   stream 1: initialisation draws
 *   uniform   : one block -> ((o0<<32|o1) >> 11) * 2^-53          in [0,1)
 *   normal x2 : one block -> u1 = (((o0<<32|o1)>>11)+1) * 2^-53   in (0,1]
 *                            u2 = ((o2<<32|o3)>>11) * 2^-53
 *               Box-Muller: r = sqrt(-2 ln u1), (r cos 2pi u2, r sin 2pi u2)
 *   momentum of D dims uses ceil(D/2) consecutive blocks; dims 2j, 2j+1
 *   take the pair of block j.
 */
#ifndef GNUTS_ORACLE_PHILOX_H
#define GNUTS_ORACLE_PHILOX_H
#include <stdint.h>
#include <math.h>

static inline void orc_philox_impl(const uint32_t c[4], const uint32_t k[2], uint32_t o[4]) {
  uint32_t x0 = c[0], x1 = c[1], x2 = c[2], x3 = c[3];
  uint32_t k0 = k[0], k1 = k[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * x0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * x2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t y0 = hi1 ^ x1 ^ k0;
    uint32_t y1 = lo1;
    uint32_t y2 = hi0 ^ x3 ^ k1;
    uint32_t y3 = lo0;
    x0 = y0; x1 = y1; x2 = y2; x3 = y3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  o[0] = x0; o[1] = x1; o[2] = x2; o[3] = x3;
}

typedef struct {
  uint32_t seed, chain, stream;
  uint64_t n;
} orc_rng;

static inline void orc_block(const orc_rng* g, uint64_t n, uint32_t o[4]) {
  uint32_t c[4] = {(uint32_t)n, (uint32_t)(n >> 32), g->stream, 0u};
  uint32_t k[2] = {g->seed, g->chain};
  orc_philox_impl(c, k, o);
}

static inline double orc_next_uniform(orc_rng* g) {
  uint32_t o[4];
  orc_block(g, g->n++, o);
  uint64_t x = ((uint64_t)o[0] << 32) | o[1];
  return (double)(x >> 11) * 0x1.0p-53;
}

static inline void orc_normal_from_block(const uint32_t o[4], double* z0, double* z1) {
  uint64_t a = ((uint64_t)o[0] << 32) | o[1];
  uint64_t b = ((uint64_t)o[2] << 32) | o[3];
  double u1 = (double)((a >> 11) + 1) * 0x1.0p-53;
  double u2 = (double)(b >> 11) * 0x1.0p-53;
  double r = sqrt(-2.0 * log(u1));
  double t = 6.283185307179586476925286766559 * u2;
  *z0 = r * cos(t);
  *z1 = r * sin(t);
}

/* D standard normals, ceil(D/2) blocks */
static inline void orc_next_normals(orc_rng* g, int D, double* z) {
  for (int j = 0; 2 * j < D; ++j) {
    uint32_t o[4];
    orc_block(g, g->n + (uint64_t)j, o);
    double a, b;
    orc_normal_from_block(o, &a, &b);
    z[2 * j] = a;
    if (2 * j + 1 < D) z[2 * j + 1] = b;
  }
  g->n += (uint64_t)((D + 1) / 2);
}

#endif

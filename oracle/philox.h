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
 *   normal x2 : one block -> FP32 Box-Muller from o0, o1 (orc_normal_from_block)
 *   momentum of D dims uses ceil(D/2) consecutive blocks; dims 2j, 2j+1
 *   take the pair of block j.
 */
#ifndef GNUTS_ORACLE_PHILOX_H
#define GNUTS_ORACLE_PHILOX_H
#include <stdint.h>
#include <math.h>
#include <string.h>

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

/* FP32 Box-Muller from explicit correctly rounded steps (the oracle is built
 * with -ffp-contract=off so that only the written fmaf calls fuse):
 *   ln x  = e ln2 + s (2 + z (2/3 + z (2/5 + z (2/7 + z 2/9)))),
 *           s = (m-1)/(m+1), z = s^2, x = m 2^e with m in [sqrt(1/2), sqrt(2))
 *   sin a = a (1 - z/6 + z^2/120 - z^3/5040 + z^4/362880)        a in [0, pi/4]
 *   cos a = 1 + z (-1/2 + z (1/24 + z (-1/720 + z (1/40320 - z/3628800))))
 *   2 pi u2 = k pi/2 + phi, k = floor(4 u2), phi folded into [0, pi/4]. */
static inline float orc_bm_log(float x) {
  uint32_t bits;
  memcpy(&bits, &x, 4);
  int e = (int)(bits >> 23) - 127;
  uint32_t mb = (bits & 0x7FFFFFu) | 0x3F800000u;
  float m;
  memcpy(&m, &mb, 4);
  if (m > 1.41421356237309505f) {
    m = m * 0.5f;
    e += 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float z = s * s;
  float p = fmaf(z, 0.222222222222222222f, 0.285714285714285714f);
  p = fmaf(z, p, 0.4f);
  p = fmaf(z, p, 0.666666666666666667f);
  p = fmaf(z, p, 2.0f);
  return fmaf((float)e, 0.693147180559945309f, s * p);
}
static inline void orc_bm_quarter(float a, float* s, float* c) {
  const float z = a * a;
  float ps = fmaf(z, 2.75573192239858907e-6f, -1.98412698412698413e-4f);
  ps = fmaf(z, ps, 8.33333333333333333e-3f);
  ps = fmaf(z, ps, -0.166666666666666667f);
  ps = fmaf(z, ps, 1.0f);
  *s = a * ps;
  float pc = fmaf(z, -2.75573192239858907e-7f, 2.48015873015873016e-5f);
  pc = fmaf(z, pc, -1.38888888888888889e-3f);
  pc = fmaf(z, pc, 4.16666666666666667e-2f);
  pc = fmaf(z, pc, -0.5f);
  *c = fmaf(z, pc, 1.0f);
}
static inline void orc_normal_from_block(const uint32_t o[4], double* z0, double* z1) {
  const float u1 = (float)(((double)o[0] + 1.0) * 0x1.0p-32);
  const float u2 = (float)(o[1] >> 8) * 0x1.0p-24f;
  const float r = sqrtf(-2.0f * orc_bm_log(u1));
  const float t = 4.0f * u2;
  const float k = floorf(t);
  const float f = t - k;
  float s, c;
  if (f <= 0.5f) orc_bm_quarter(f * 1.57079632679489662f, &s, &c);
  else orc_bm_quarter((1.0f - f) * 1.57079632679489662f, &c, &s);
  float cs, sn;
  switch ((int)k) {
    case 0: cs = c; sn = s; break;
    case 1: cs = -s; sn = c; break;
    case 2: cs = -c; sn = -s; break;
    default: cs = s; sn = -c; break;
  }
  *z0 = (double)(r * cs);
  *z1 = (double)(r * sn);
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

// Counter-based Philox-4x32-10 random numbers for the device sampler.
//
// Replaces the per-chain boost::ecuyer1988 generator that the reference's
// services create (stan::services::util::create_rng, called for every chain
// by the hmc_nuts_* services; src/cmdstan/command.hpp:657-688).  Bitwise RNG
// parity with CmdStan is neither possible nor required; what is fixed is the
// schedule below, which the CPU oracle restates independently:
//   key     = {seed, chain_id}
//   counter = {lo32(n), hi32(n), stream, 0}; n is the per-stream draw index
//   stream 0: sampler (jitter, momentum, direction, multinomial choices)
//   stream 1: initial values
//   uniform : ((o0<<32 | o1) >> 11) * 2^-53 in [0,1)
//   normals : FP32 Box-Muller pair (r cos 2 pi u2, r sin 2 pi u2) from o0, o1
//             (bm_normal below); dims 2j and 2j+1 of a momentum take the pair
//             of block n0 + j.
#pragma once
#include <stdint.h>

namespace gnuts {

__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1, uint32_t o[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t lo0 = 0xD2511F53u * c0;
    uint32_t hi0 = __umulhi(0xD2511F53u, c0);
    uint32_t lo1 = 0xCD9E8D57u * c2;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c2);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  o[0] = c0; o[1] = c1; o[2] = c2; o[3] = c3;
}

__device__ __forceinline__ void rng_block(uint32_t seed, uint32_t chain, uint32_t stream, uint64_t n,
                                          uint32_t o[4]) {
  philox4x32_10((uint32_t)n, (uint32_t)(n >> 32), stream, 0u, seed, chain, o);
}

__device__ __forceinline__ double rng_uniform(uint32_t seed, uint32_t chain, uint32_t stream,
                                              uint64_t n) {
  uint32_t o[4];
  rng_block(seed, chain, stream, n, o);
  uint64_t x = ((uint64_t)o[0] << 32) | o[1];
  return (double)(x >> 11) * 0x1.0p-53;
}

// Normal draws: Box-Muller in FP32 from explicit correctly rounded operations
// (no library math, no contraction), so every IEEE-conforming implementation
// of the same steps returns the same bits:
//   u1 = float((o0 + 1) 2^-32) in (0, 1], u2 = (o1 >> 8) 2^-24 in [0, 1)
//   ln u1 = e ln2 + 2 atanh(s), s = (m-1)/(m+1), m in [sqrt(1/2), sqrt(2)),
//           atanh series to s^9 (|s| <= 0.172, truncation < 4e-10)
//   (cos, sin)(2 pi u2): quarter turn k = floor(4 u2), f = 4 u2 - k, angle
//           f pi/2 folded to [0, pi/4] and Taylor series to a^9 / a^10
//   z0 = r cos, z1 = r sin, r = sqrt(-2 ln u1)
__device__ __forceinline__ float bm_log(float x) {
  uint32_t bits = __float_as_uint(x);
  int e = (int)(bits >> 23) - 127;
  float m = __uint_as_float((bits & 0x7FFFFFu) | 0x3F800000u);
  if (m > 1.41421356237309505f) {
    m = __fmul_rn(m, 0.5f);
    e += 1;
  }
  const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
  const float z = __fmul_rn(s, s);
  float p = __fmaf_rn(z, 0.222222222222222222f, 0.285714285714285714f);
  p = __fmaf_rn(z, p, 0.4f);
  p = __fmaf_rn(z, p, 0.666666666666666667f);
  p = __fmaf_rn(z, p, 2.0f);
  return __fmaf_rn((float)e, 0.693147180559945309f, __fmul_rn(s, p));
}
__device__ __forceinline__ void bm_sincos_quarter(float a, float* s, float* c) {
  const float z = __fmul_rn(a, a);
  float ps = __fmaf_rn(z, 2.75573192239858907e-6f, -1.98412698412698413e-4f);
  ps = __fmaf_rn(z, ps, 8.33333333333333333e-3f);
  ps = __fmaf_rn(z, ps, -0.166666666666666667f);
  ps = __fmaf_rn(z, ps, 1.0f);
  *s = __fmul_rn(a, ps);
  float pc = __fmaf_rn(z, -2.75573192239858907e-7f, 2.48015873015873016e-5f);
  pc = __fmaf_rn(z, pc, -1.38888888888888889e-3f);
  pc = __fmaf_rn(z, pc, 4.16666666666666667e-2f);
  pc = __fmaf_rn(z, pc, -0.5f);
  *c = __fmaf_rn(z, pc, 1.0f);
}
__device__ __forceinline__ double bm_normal(const uint32_t o[4], int component) {
  const float u1 = (float)(((double)o[0] + 1.0) * 0x1.0p-32);
  const float u2 = (float)(o[1] >> 8) * 0x1.0p-24f;
  const float r = __fsqrt_rn(__fmul_rn(-2.0f, bm_log(u1)));
  const float t = __fmul_rn(4.0f, u2);
  const float k = floorf(t);
  float f = __fsub_rn(t, k);
  float s, c;
  if (f <= 0.5f) {
    bm_sincos_quarter(__fmul_rn(f, 1.57079632679489662f), &s, &c);
  } else {
    bm_sincos_quarter(__fmul_rn(__fsub_rn(1.0f, f), 1.57079632679489662f), &c, &s);
  }
  const int q = (int)k;
  float cs, sn;  // cos and sin of 2 pi u2
  if (q == 0) { cs = c; sn = s; }
  else if (q == 1) { cs = -s; sn = c; }
  else if (q == 2) { cs = -c; sn = -s; }
  else { cs = s; sn = -c; }
  return (double)__fmul_rn(r, component ? sn : cs);
}

// component (0 or 1) of the Box-Muller pair of block n
__device__ __forceinline__ double rng_normal(uint32_t seed, uint32_t chain, uint32_t stream,
                                             uint64_t n, int component) {
  uint32_t o[4];
  rng_block(seed, chain, stream, n, o);
  return bm_normal(o, component);
}

}  // namespace gnuts

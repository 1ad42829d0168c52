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
//   normals : u1 = (((o0<<32|o1)>>11) + 1) 2^-53 in (0,1], u2 = ((o2<<32|o3)>>11) 2^-53,
//             Box-Muller pair (r cos 2 pi u2, r sin 2 pi u2), r = sqrt(-2 ln u1);
//             dims 2j and 2j+1 of a momentum take the pair of block n0 + j.
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

// component (0 or 1) of the Box-Muller pair of block n
__device__ __forceinline__ double rng_normal(uint32_t seed, uint32_t chain, uint32_t stream,
                                             uint64_t n, int component) {
  uint32_t o[4];
  rng_block(seed, chain, stream, n, o);
  uint64_t a = ((uint64_t)o[0] << 32) | o[1];
  uint64_t b = ((uint64_t)o[2] << 32) | o[3];
  double u1 = (double)((a >> 11) + 1) * 0x1.0p-53;
  double u2 = (double)(b >> 11) * 0x1.0p-53;
  double r = sqrt(-2.0 * log(u1));
  double t = 6.283185307179586476925286766559 * u2;
  return component ? r * sin(t) : r * cos(t);
}

}  // namespace gnuts

// stansummary statistics on the GPU: one CTA per quantity.
//
// The same statistics and the same algorithms as the host version
// (summary.cpp, which restates what src/cmdstan/stansummary_helper.hpp:397-428
// obtains from stan::mcmc::chainset): mean, MCSE of the mean (from the ESS of
// the raw, unsplit chains), SD, MAD, type-7 quantiles, split rank-normalised
// bulk and tail ESS (Geyer truncation) and R-hat = max(bulk, folded).  What
// changes is where the time goes: the host sorts each quantity's pooled draws
// four times with std::sort; here a CTA sorts them twice (draws, then their
// distances to the median) with an LSD radix sort in global memory and
// derives quantiles, ranks (average ranks for ties), normal scores and the
// MAD from those two orders; the autocovariances behind every ESS are
// CTA-wide reductions, eight lags per pass over the draws.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>
#include "../../include/gnuts.h"

namespace gnuts {
namespace {

constexpr int ST = 1024;  // threads per CTA
constexpr int NW = ST / 32;
constexpr int LAGS = 8;   // autocovariance lags per pass

// Wichura, "Algorithm AS 241", PPND16 (the same coefficients as the host).
__device__ double ppnd16_d(double p) {
  const double q = p - 0.5;
  if (fabs(q) <= 0.425) {
    const double r = 0.180625 - q * q;
    return q *
           (((((((2509.0809287301226727 * r + 33430.575583588128105) * r + 67265.770927008700853) * r +
                45921.953931549871457) * r + 13731.693765509461125) * r + 1971.5909503065514427) * r +
             133.14166789178437745) * r + 3.387132872796366608) /
           (((((((5226.495278852545925 * r + 28729.085735721942674) * r + 39307.89580009271061) * r +
                21213.794301586595867) * r + 5394.1960214247511077) * r + 687.1870074920579083) * r +
             42.313330701600911252) * r + 1.0);
  }
  double r = q < 0 ? p : 1.0 - p;
  if (r <= 0) return q < 0 ? -INFINITY : INFINITY;
  r = sqrt(-log(r));
  double v;
  if (r <= 5.0) {
    r -= 1.6;
    v = (((((((7.7454501427834140764e-4 * r + 0.0227238449892691845833) * r + 0.24178072517745061177) * r +
             1.27045825245236838258) * r + 3.64784832476320460504) * r + 5.7694972214606914055) * r +
          4.6303378461565452959) * r + 1.42343711074968357734) /
        (((((((1.05075007164441684324e-9 * r + 5.475938084995344946e-4) * r + 0.0151986665636164571966) * r +
             0.14810397642748007459) * r + 0.68976733498510000455) * r + 1.6763848301838038494) * r +
          2.05319162663775882187) * r + 1.0);
  } else {
    r -= 5.0;
    v = (((((((2.01033439929228813265e-7 * r + 2.71155556874348757815e-5) * r + 0.0012426609473880784386) * r +
             0.026532189526576123093) * r + 0.29656057182850489123) * r + 1.7848265399172913358) * r +
          5.4637849111641143699) * r + 6.6579046435011037772) /
        (((((((2.04426310338993978564e-15 * r + 1.4215117583164458887e-7) * r + 1.8463183175100546818e-5) * r +
             7.868691311456132591e-4) * r + 0.0148753612908506148525) * r + 0.13692988092273580531) * r +
          0.59983220655588793769) * r + 1.0);
  }
  return q < 0 ? -v : v;
}

struct Shared {
  double red[NW][LAGS];
  unsigned hist[256];
  unsigned offset[256];
  unsigned total[256];
  unsigned wc[NW][256];
  unsigned long long flag;
  long long scan[NW];
  long long carry;
};

// CTA sum of LAGS values per thread (every thread gets the result)
__device__ void block_sum(Shared& sh, double* v, int nv) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = 0; j < nv; ++j)
    for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
  __syncthreads();
  if (lane == 0)
    for (int j = 0; j < nv; ++j) sh.red[w][j] = v[j];
  __syncthreads();
  for (int j = 0; j < nv; ++j) {
    double t = 0;
    for (int k = 0; k < NW; ++k) t += sh.red[k][j];  // fixed order: identical on every thread
    v[j] = t;
  }
  __syncthreads();
}

__device__ __forceinline__ unsigned long long dkey(double x) {
  if (x == 0.0) x = 0.0;  // -0 and +0 compare equal: one key
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dval(unsigned long long k) {
  const unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}

// stable LSD radix sort of (key, val) pairs by the CTA; the sorted pairs end
// in (k0, v0) (k1, v1 are scratch).  Digits where every key agrees are skipped.
__device__ void radix_sort(Shared& sh, unsigned long long* k0, unsigned* v0, unsigned long long* k1, unsigned* v1,
                           long long n) {
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  unsigned long long *ka = k0, *kb = k1;
  unsigned *va = v0, *vb = v1;
  for (int pass = 0; pass < 8; ++pass) {
    const int shift = 8 * pass;
    if (tid < 256) sh.hist[tid] = 0;
    __syncthreads();
    for (long long i = tid; i < n; i += ST) atomicAdd(&sh.hist[(unsigned)(ka[i] >> shift) & 255u], 1u);
    __syncthreads();
    bool skip = false;
    if (tid == 0) {
      unsigned run = 0;
      sh.flag = 0;
      for (int d = 0; d < 256; ++d) {
        if (sh.hist[d] == (unsigned long long)n) sh.flag = 1;
        sh.offset[d] = run;
        run += sh.hist[d];
      }
    }
    __syncthreads();
    skip = sh.flag != 0;
    if (skip) continue;
    for (long long base = 0; base < n; base += ST) {
      const long long i = base + tid;
      const bool valid = i < n;
      const unsigned long long key = valid ? ka[i] : 0ull;
      const unsigned val = valid ? va[i] : 0u;
      const unsigned d = valid ? ((unsigned)(key >> shift) & 255u) : 256u;
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      const unsigned lt = (1u << lane) - 1u;
      const unsigned rank = __popc(peers & lt);
      if (valid && rank == 0) sh.wc[w][d] = __popc(peers);
      __syncthreads();
      if (tid < 256) {
        unsigned run = 0;
        for (int k = 0; k < NW; ++k) {
          const unsigned t = sh.wc[k][tid];
          sh.wc[k][tid] = run;
          run += t;
        }
        sh.total[tid] = run;
      }
      __syncthreads();
      if (valid) {
        const unsigned pos = sh.offset[d] + sh.wc[w][d] + rank;
        kb[pos] = key;
        vb[pos] = val;
      }
      __syncthreads();
      if (tid < 256) {
        sh.offset[tid] += sh.total[tid];
        for (int k = 0; k < NW; ++k) sh.wc[k][tid] = 0;
      }
      __syncthreads();
    }
    unsigned long long* tk = ka;
    ka = kb;
    kb = tk;
    unsigned* tv = va;
    va = vb;
    vb = tv;
  }
  // the result must end in (k0, v0)
  if (ka != k0) {
    for (long long i = threadIdx.x; i < n; i += ST) {
      k0[i] = ka[i];
      v0[i] = va[i];
    }
  }
  __syncthreads();
}

// inclusive CTA scan helpers over chunks of ST elements with a carry
__device__ long long block_scan_sum(Shared& sh, long long v) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh.scan[w] = x;
  __syncthreads();
  if (w == 0) {
    long long s = sh.scan[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    sh.scan[lane] = s;
  }
  __syncthreads();
  const long long r = x + (w ? sh.scan[w - 1] : 0) + sh.carry;
  __syncthreads();
  if (threadIdx.x == ST - 1) sh.carry = r;
  __syncthreads();
  return r;
}
__device__ long long block_scan_max(Shared& sh, long long v) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x = x > y ? x : y;
  }
  if (lane == 31) sh.scan[w] = x;
  __syncthreads();
  if (w == 0) {
    long long s = sh.scan[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s = s > y ? s : y;
    }
    sh.scan[lane] = s;
  }
  __syncthreads();
  long long r = w ? (x > sh.scan[w - 1] ? x : sh.scan[w - 1]) : x;
  r = r > sh.carry ? r : sh.carry;
  __syncthreads();
  if (threadIdx.x == ST - 1) sh.carry = r;
  __syncthreads();
  return r;
}

// Normal scores of the pooled average ranks of the included elements of a
// sorted order (k: sorted keys, v: original positions).  Elements whose
// position is excluded (the middle draw of odd-length chains, which the split
// drops) take no rank.  Writes z[position].  tmp: n longs of scratch.
template <class Incl>
__device__ void rank_scores(Shared& sh, const unsigned long long* k, const unsigned* v, long long n, Incl incl,
                            long long* tmp, double* z) {
  const int tid = threadIdx.x;
  // 1. compact the included elements (stable) into tmp as sorted-position indices
  if (tid == 0) sh.carry = 0;
  __syncthreads();
  long long m = 0;
  for (long long base = 0; base < n; base += ST) {
    const long long i = base + tid;
    const int f = (i < n && incl(v[i])) ? 1 : 0;
    const long long c = block_scan_sum(sh, f);
    if (f) tmp[c - 1] = i;
    m = sh.carry;
  }
  __syncthreads();
  // 2. run starts among the included (forward max-scan of boundary positions)
  //    written over tmp's high half: store start in the sign-free upper bits
  //    of a second pass; keep it simple with a second array region
  long long* start = tmp + n;
  if (tid == 0) sh.carry = 0;
  __syncthreads();
  for (long long base = 0; base < m; base += ST) {
    const long long j = base + tid;
    long long b = 0;
    if (j < m) b = (j == 0 || k[tmp[j]] != k[tmp[j - 1]]) ? j : 0;
    const long long s = block_scan_max(sh, b);
    if (j < m) start[j] = s;
  }
  __syncthreads();
  // 3. run ends: scan the reversed order for the next boundary
  if (tid == 0) sh.carry = -(long long)m;
  __syncthreads();
  for (long long base = 0; base < m; base += ST) {
    const long long j = m - 1 - (base + tid);  // walking backwards
    long long b = -(long long)m;
    if (j >= 0) b = (j == m - 1 || k[tmp[j]] != k[tmp[j + 1]]) ? -(j + 1) : -(long long)m;
    const long long e = -block_scan_max(sh, b);  // smallest end >= j + 1 among boundaries at or after j
    if (j >= 0) {
      const double rank = 0.5 * (double)(start[j] + 1 + e);
      z[v[tmp[j]]] = ppnd16_d((rank - 0.375) / ((double)m + 0.25));
    }
  }
  __syncthreads();
}

// Effective sample size of the sequences s = 0..M-1 of length len, element t
// of sequence s read by get(s, t) (Geyer truncation, as ess_of on the host).
// cm: M doubles, rho: len + 2 doubles of scratch.
template <class Get>
__device__ double ess_dev(Shared& sh, int M, int len, Get get, double* cm, double* rho) {
  const int tid = threadIdx.x;
  if (len < 4) return NAN;
  // sequence means (one warp per sequence, fixed order)
  const int lane = tid & 31, w = tid >> 5;
  for (int s = w; s < M; s += NW) {
    double a = 0;
    for (int t = lane; t < len; t += 32) a += get(s, t);
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) cm[s] = a / len;
  }
  __syncthreads();
  // constant check
  const double first = get(0, 0);
  double nc[1] = {0};
  const long long total_n = (long long)M * len;
  for (long long e = tid; e < total_n; e += ST)
    if (get((int)(e / len), (int)(e % len)) != first) nc[0] += 1;
  block_sum(sh, nc, 1);
  if (nc[0] == 0) return NAN;
  // variance of the sequence means
  double mm[1] = {0};
  for (int s = tid; s < M; s += ST) mm[0] += cm[s];
  block_sum(sh, mm, 1);
  const double mbar = mm[0] / M;
  double vm[1] = {0};
  for (int s = tid; s < M; s += ST) vm[0] += (cm[s] - mbar) * (cm[s] - mbar);
  block_sum(sh, vm, 1);
  const double var_cm = M > 1 ? vm[0] / (M - 1) : 0.0;
  // autocovariances, LAGS per pass, cached in rho[] as they are computed
  int have = 0;
  auto acov = [&](int k) -> double {
    while (have <= k) {
      double a[LAGS];
      for (int j = 0; j < LAGS; ++j) a[j] = 0;
      for (long long e = tid; e < total_n; e += ST) {
        const int s = (int)(e / len), t = (int)(e % len);
        const double x0 = get(s, t) - cm[s];
        for (int j = 0; j < LAGS; ++j) {
          const int kk = have + j;
          if (t + kk < len) a[j] += x0 * (get(s, t + kk) - cm[s]);
        }
      }
      block_sum(sh, a, LAGS);
      for (int j = 0; j < LAGS && have + j < len + 2; ++j) rho[have + j] = a[j] / len / M;
      have += LAGS;
    }
    return rho[k];
  };
  const double a0 = acov(0);
  const double mean_var = a0 * len / (len - 1.0);
  double var_plus = mean_var * (len - 1.0) / len;
  if (M > 1) var_plus += var_cm;
  auto rho_at = [&](int k) { return 1.0 - (mean_var - acov(k)) / var_plus; };
  // Geyer's initial positive / monotone sequence on the rho values (every
  // thread runs the same scalar recursion on identical values)
  double r0 = 1.0, r1 = rho_at(1);
  // rho values used by the truncation live in a separate small array: reuse
  // cm[M..] would alias; keep them in registers-free scratch after the acov cache
  double* rr = rho + (len + 2 + LAGS);
  for (int k = 0; k < len + 2; ++k)
    if (k > 1 && tid == 0) rr[k] = 0.0;
  __syncthreads();
  int t = 0;
  double even = r0, odd = r1;
  if (tid == 0) {
    rr[0] = even;
    rr[1] = odd;
  }
  __syncthreads();
  while (t < len - 5 && !isnan(even + odd) && even + odd > 0) {
    t += 2;
    even = rho_at(t);
    odd = rho_at(t + 1);
    if (even + odd >= 0 && tid == 0) {
      rr[t] = even;
      rr[t + 1] = odd;
    }
    __syncthreads();
  }
  const int max_t = t;
  if (even > 0 && tid == 0) rr[max_t] = even;
  __syncthreads();
  double tau = 0;
  if (tid == 0) {
    for (int u = 2; u <= max_t - 2; u += 2) {
      const double prev = rr[u - 2] + rr[u - 1];
      if (rr[u] + rr[u + 1] > prev) {
        rr[u] = prev / 2;
        rr[u + 1] = rr[u];
      }
    }
    tau = -1.0 + rr[max_t];
    for (int k = 0; k < max_t; ++k) tau += 2.0 * rr[k];
    const double total = (double)M * len;
    tau = fmax(tau, 1.0 / log10(total));
    sh.red[0][0] = total / tau;
  }
  __syncthreads();
  const double ess = sh.red[0][0];
  __syncthreads();
  return ess;
}

// R-hat of M sequences (as rhat_of on the host)
template <class Get>
__device__ double rhat_dev(Shared& sh, int M, int len, Get get, double* cm, double* cv) {
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  for (int s = w; s < M; s += NW) {
    double a = 0;
    for (int t = lane; t < len; t += 32) a += get(s, t);
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    const double mu = a / len;
    double b = 0;
    for (int t = lane; t < len; t += 32) b += (get(s, t) - mu) * (get(s, t) - mu);
    for (int o = 16; o > 0; o >>= 1) b += __shfl_xor_sync(0xffffffffu, b, o);
    if (lane == 0) {
      cm[s] = mu;
      cv[s] = b / (len - 1);
    }
  }
  __syncthreads();
  double a[2] = {0, 0};
  for (int s = tid; s < M; s += ST) {
    a[0] += cm[s];
    a[1] += cv[s];
  }
  block_sum(sh, a, 2);
  const double mbar = a[0] / M, within = a[1] / M;
  double b[1] = {0};
  for (int s = tid; s < M; s += ST) b[0] += (cm[s] - mbar) * (cm[s] - mbar);
  block_sum(sh, b, 1);
  const double between = len * (b[0] / (M - 1));
  return sqrt((between / within + len - 1.0) / len);
}

struct ColJob {
  const double* x;    // [M][n] draws of this quantity
  double* out;        // 7 + np values
  // scratch
  unsigned long long *k0, *k1;
  unsigned *v0, *v1;
  long long* tmp;     // 2 S
  double* z;          // S
  double* seq;        // 2 (2M) + 3 (n + 2 + LAGS) doubles
};

__global__ void __launch_bounds__(ST, 1) k_summary(const ColJob* jobs, int M, int n, const double* probs, int np) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Shared& sh = *reinterpret_cast<Shared*>(smem_raw);
  const ColJob J = jobs[blockIdx.x];
  const int tid = threadIdx.x;
  const long long S = (long long)M * n;
  const int h = n / 2;
  const double* x = J.x;
  double* cm = J.seq;
  double* cv = J.seq + 2 * M;
  double* rho = J.seq + 4 * M;
  for (int i = tid; i < 256; i += ST) sh.hist[i] = 0;
  for (int i = tid; i < NW * 256; i += ST) (&sh.wc[0][0])[i] = 0;
  __syncthreads();
  // mean and SD of all draws
  double s1[1] = {0};
  for (long long e = tid; e < S; e += ST) s1[0] += x[e];
  block_sum(sh, s1, 1);
  const double mu = s1[0] / S;
  double s2[1] = {0};
  for (long long e = tid; e < S; e += ST) s2[0] += (x[e] - mu) * (x[e] - mu);
  block_sum(sh, s2, 1);
  const double sd = sqrt(s2[0] / (S - 1));
  // MCSE from the ESS of the raw chains
  const double ess_raw = ess_dev(sh, M, n, [&](int s, int t) { return x[(size_t)s * n + t]; }, cm, rho);
  // sort all draws: quantiles and the median
  for (long long e = tid; e < S; e += ST) {
    J.k0[e] = dkey(x[e]);
    J.v0[e] = (unsigned)e;
  }
  __syncthreads();
  radix_sort(sh, J.k0, J.v0, J.k1, J.v1, S);
  auto quant = [&](const unsigned long long* ks, double p) {
    const double hh = (S - 1) * p;
    const long long lo = (long long)floor(hh);
    const long long hi = lo + 1 < S ? lo + 1 : S - 1;
    const double a = dval(ks[lo]), b = dval(ks[hi]);
    return a + (hh - lo) * (b - a);
  };
  const double med = quant(J.k0, 0.5), q05 = quant(J.k0, 0.05), q95 = quant(J.k0, 0.95);
  if (tid == 0) {
    J.out[0] = mu;
    J.out[1] = sd / sqrt(ess_raw);
    J.out[2] = sd;
    for (int k = 0; k < np; ++k) J.out[4 + k] = quant(J.k0, probs[k]);
  }
  // split sequences: s = 2m (first h draws) or 2m + 1 (last h draws)
  auto split_pos = [&](int s, int t) -> size_t { return (size_t)(s >> 1) * n + (size_t)(t + ((s & 1) ? n - h : 0)); };
  auto included = [&](unsigned e) { return (n % 2 == 0) || (int)(e % n) != h; };
  // bulk: normal scores of the pooled ranks of the split draws
  rank_scores(sh, J.k0, J.v0, S, included, J.tmp, J.z);
  const double* z = J.z;
  const double ess_bulk = ess_dev(sh, 2 * M, h, [&](int s, int t) { return z[split_pos(s, t)]; }, cm, rho);
  const double rhat_bulk = rhat_dev(sh, 2 * M, h, [&](int s, int t) { return z[split_pos(s, t)]; }, cm, cv);
  // tail: indicators of the 5 % and 95 % quantiles on the split draws
  const double e05 = ess_dev(sh, 2 * M, h, [&](int s, int t) { return x[split_pos(s, t)] <= q05 ? 1.0 : 0.0; }, cm, rho);
  const double e95 = ess_dev(sh, 2 * M, h, [&](int s, int t) { return x[split_pos(s, t)] <= q95 ? 1.0 : 0.0; }, cm, rho);
  // folded draws |x - median|: MAD over all draws, folded R-hat on split ranks
  for (long long e = tid; e < S; e += ST) {
    J.k0[e] = dkey(fabs(x[e] - med));
    J.v0[e] = (unsigned)e;
  }
  __syncthreads();
  radix_sort(sh, J.k0, J.v0, J.k1, J.v1, S);
  const double mad = 1.4826 * quant(J.k0, 0.5);
  rank_scores(sh, J.k0, J.v0, S, included, J.tmp, J.z);
  const double rhat_fold = rhat_dev(sh, 2 * M, h, [&](int s, int t) { return z[split_pos(s, t)]; }, cm, cv);
  if (tid == 0) {
    J.out[3] = mad;
    J.out[4 + np] = ess_bulk;
    J.out[5 + np] = fmin(e05, e95);
    J.out[6 + np] = fmax(rhat_bulk, rhat_fold);
  }
}

}  // namespace
}  // namespace gnuts

using namespace gnuts;

extern "C" int gnuts_summary_columns_gpu(const double* draws, int n_chains, int n_iter, int n_cols,
                                         int64_t stride_chain, int64_t stride_iter, const int* cols,
                                         const double* probs, int n_probs, double* out) {
  if (!draws || !out || !cols || n_chains < 1 || n_iter < 4 || n_cols < 0 || n_probs < 0 ||
      (n_probs > 0 && !probs))
    return GNUTS_ERR_ARGUMENT;
  if ((long long)n_chains * n_iter >= (1ll << 31)) return GNUTS_ERR_ARGUMENT;
  if (n_cols == 0) return GNUTS_OK;
  nvtxRangePushA("gnuts.summary.gpu");
  struct Pop { ~Pop() { nvtxRangePop(); } } pop;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GNUTS_ERR_CUDA;
  const int M = n_chains, n = n_iter;
  const long long S = (long long)M * n;
  const int np = n_probs;
  // columns per launch: bounded device memory (about 48 bytes per draw)
  const int batch = (int)std::max<long long>(1, std::min<long long>(n_cols, (6ll << 30) / (S * 48)));
  const size_t per_seq = 4 * (size_t)M + 3 * ((size_t)n + 2 + LAGS);
  std::vector<double> hx((size_t)batch * S);
  double *dx = nullptr, *dz = nullptr, *dseq = nullptr, *dout = nullptr, *dprobs = nullptr;
  unsigned long long *dk0 = nullptr, *dk1 = nullptr;
  unsigned *dv0 = nullptr, *dv1 = nullptr;
  long long* dtmp = nullptr;
  ColJob* djobs = nullptr;
  int rc = GNUTS_OK;
  auto ok = [&](cudaError_t e) {
    if (e != cudaSuccess && rc == GNUTS_OK) rc = GNUTS_ERR_CUDA;
    return e == cudaSuccess;
  };
  if (ok(cudaMalloc(&dx, sizeof(double) * batch * S)) && ok(cudaMalloc(&dz, sizeof(double) * batch * S)) &&
      ok(cudaMalloc(&dseq, sizeof(double) * batch * per_seq)) &&
      ok(cudaMalloc(&dout, sizeof(double) * batch * (7 + np))) &&
      ok(cudaMalloc(&dprobs, sizeof(double) * std::max(1, np))) &&
      ok(cudaMalloc(&dk0, sizeof(unsigned long long) * batch * S)) &&
      ok(cudaMalloc(&dk1, sizeof(unsigned long long) * batch * S)) && ok(cudaMalloc(&dv0, sizeof(unsigned) * batch * S)) &&
      ok(cudaMalloc(&dv1, sizeof(unsigned) * batch * S)) && ok(cudaMalloc(&dtmp, sizeof(long long) * 2 * batch * S)) &&
      ok(cudaMalloc(&djobs, sizeof(ColJob) * batch))) {
    if (np) ok(cudaMemcpy(dprobs, probs, sizeof(double) * np, cudaMemcpyHostToDevice));
    ok(cudaFuncSetAttribute(k_summary, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Shared)));
    std::vector<ColJob> jobs(batch);
    for (int c0 = 0; c0 < n_cols && rc == GNUTS_OK; c0 += batch) {
      const int nb = std::min(batch, n_cols - c0);
      for (int j = 0; j < nb; ++j) {
        const double* src = draws + cols[c0 + j];
        double* dst = hx.data() + (size_t)j * S;
        for (int m = 0; m < M; ++m)
          for (int i = 0; i < n; ++i) dst[(size_t)m * n + i] = src[m * stride_chain + i * stride_iter];
        ColJob& J = jobs[j];
        J.x = dx + (size_t)j * S;
        J.out = dout + (size_t)j * (7 + np);
        J.k0 = dk0 + (size_t)j * S;
        J.k1 = dk1 + (size_t)j * S;
        J.v0 = dv0 + (size_t)j * S;
        J.v1 = dv1 + (size_t)j * S;
        J.tmp = dtmp + (size_t)j * 2 * S;
        J.z = dz + (size_t)j * S;
        J.seq = dseq + (size_t)j * per_seq;
      }
      if (!ok(cudaMemcpy(dx, hx.data(), sizeof(double) * nb * S, cudaMemcpyHostToDevice))) break;
      if (!ok(cudaMemcpy(djobs, jobs.data(), sizeof(ColJob) * nb, cudaMemcpyHostToDevice))) break;
      k_summary<<<nb, ST, sizeof(Shared)>>>(djobs, M, n, dprobs, np);
      if (!ok(cudaGetLastError())) break;
      if (!ok(cudaMemcpy(out + (size_t)c0 * (7 + np), dout, sizeof(double) * nb * (7 + np), cudaMemcpyDeviceToHost)))
        break;
    }
  }
  for (void* p : {(void*)dx, (void*)dz, (void*)dseq, (void*)dout, (void*)dprobs, (void*)dk0, (void*)dk1, (void*)dv0,
                  (void*)dv1, (void*)dtmp, (void*)djobs})
    if (p) cudaFree(p);
  return rc;
}

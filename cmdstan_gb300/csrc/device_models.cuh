// Warp-level log densities and hand-written adjoints on the device.
//
// Each function replaces, for one built-in model, what the stanc-generated
// log_prob plus Stan Math's reverse-mode `var` tape compute through
// stan::model::log_prob_grad<true, jacobian> (contract visible at
// src/cmdstan/command_helper.hpp:589-593): lp with `propto` (parameter-free
// terms dropped) and, when `jac`, the log-Jacobian of the constraining
// transforms; the gradient is on the unconstrained scale.
//
// One warp evaluates one point.  Lane l owns vector elements l, l+32, ...
// Reductions use an xor butterfly, which gives bitwise-identical results on
// every lane, so the scalar state that all lanes carry stays lane-uniform.
#pragma once
#include "internal.h"

namespace gnuts {

#define GN_FULL 0xffffffffu

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(GN_FULL, v, o);
  return v;
}
__device__ __forceinline__ bool wall(bool p) { return __all_sync(GN_FULL, p); }

// Team primitives.  A team of TW threads advances one chain: one warp
// (TW = 32), or the whole CTA (TW a multiple of 32 up to 1024).  Every
// thread of the team receives the same bits: the warp butterfly combines
// symmetric pairs, and the per-warp values are added by every thread in warp
// order.  TW = 32 is exactly the warp code.
template <int TW>
__device__ __forceinline__ void tsync() {
  if constexpr (TW == 32) __syncwarp();
  else __syncthreads();
}
template <int TW, int N>
__device__ __forceinline__ void tsum_n(double (&v)[N]) {
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = wsum(v[i]);
  if constexpr (TW > 32) {
    constexpr int NW = TW / 32;
    __shared__ double red[N * NW];
    __syncthreads();  // earlier readers of red are done
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
      for (int i = 0; i < N; ++i) red[i * NW + (threadIdx.x >> 5)] = v[i];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < N; ++i) {
      double t = 0;
#pragma unroll
      for (int w = 0; w < NW; ++w) t += red[i * NW + w];
      v[i] = t;
    }
  }
}
template <int TW>
__device__ __forceinline__ double tsum(double v) {
  double a[1] = {v};
  tsum_n<TW, 1>(a);
  return a[0];
}
template <int TW>
__device__ __forceinline__ bool tall(bool p) {
  if constexpr (TW == 32) return wall(p);
  else return __syncthreads_and(p) != 0;
}

__device__ __forceinline__ double log1p_exp(double a) {
  return a > 0 ? a + log1p(exp(-a)) : log1p(exp(a));
}
__device__ __forceinline__ double inv_logit(double a) {
  if (a >= 0) return 1.0 / (1.0 + exp(-a));
  double e = exp(a);
  return e / (1.0 + e);
}

// ---- bernoulli: theta ~ beta(1,1), y ~ bernoulli(theta), theta = inv_logit(u)
static __device__ __noinline__ double lpg_bernoulli(const DevModel& M, const double* q, double* g, int jac, int lane) {
  double u = q[0];
  double a = M.ysum + (jac ? 1.0 : 0.0), b = (M.N - M.ysum) + (jac ? 1.0 : 0.0);
  double th = inv_logit(u);
  double lp = -a * log1p_exp(-u) - b * log1p_exp(u);
  if (lane == 0) g[0] = a * (1.0 - th) - b * th;
  return lp;
}

// ---- normal: x_k ~ normal(0, s_k)
static __device__ __noinline__ double lpg_normal(const DevModel& M, const double* q, double* g, int jac, int lane) {
  double lp = 0;
  for (int k = lane; k < M.K; k += 32) {
    double s = M.scales[k], x = q[k];
    lp += -0.5 * (x / s) * (x / s);
    g[k] = -x / (s * s);
  }
  return wsum(lp);
}

// ---- funnel: v ~ normal(0,3), x_k ~ normal(0, exp(v/2))
static __device__ __noinline__ double lpg_funnel(const DevModel& M, const double* q, double* g, int jac, int lane) {
  double v = q[0];
  double ev = exp(-v);
  double lp = 0, gv = 0;
  for (int k = lane; k < M.K; k += 32) {
    double x = q[1 + k];
    lp += -0.5 * v - 0.5 * x * x * ev;
    gv += -0.5 + 0.5 * x * x * ev;
    g[1 + k] = -x * ev;
  }
  lp = wsum(lp) - 0.5 * (v / 3.0) * (v / 3.0);
  gv = wsum(gv) - v / 9.0;
  if (lane == 0) g[0] = gv;
  return lp;
}

// ---- hier (eight schools, centered): [mu, theta_1..J, log tau]
static __device__ __noinline__ double lpg_hier(const DevModel& M, const double* q, double* g, int jac, int lane) {
  const int J = M.J;
  double mu = q[0], lt = q[J + 1], tau = exp(lt);
  double lp = 0, gmu = 0, glt = 0;
  for (int j = lane; j < J; j += 32) {
    double th = q[1 + j];
    double z = (th - mu) / tau;
    double e = (M.yr[j] - th) / M.sigma[j];
    lp += -lt - 0.5 * z * z - 0.5 * e * e;
    g[1 + j] = -z / tau + e / M.sigma[j];
    gmu += z / tau;
    glt += -1.0 + z * z;
  }
  lp = wsum(lp);
  gmu = wsum(gmu);
  glt = wsum(glt);
  double t5 = tau / 5.0;
  lp += -0.5 * (mu / 5.0) * (mu / 5.0) - log1p(t5 * t5) + (jac ? lt : 0.0);
  gmu += -mu / 25.0;
  glt += -2.0 * t5 * t5 / (1.0 + t5 * t5) + (jac ? 1.0 : 0.0);
  if (lane == 0) {
    g[0] = gmu;
    g[J + 1] = glt;
  }
  return lp;
}

// ---- logistic (warp version; the batched tensor-core kernels live in grad_logistic.cu)
// [alpha, beta_1..D]; lanes own beta elements, rows are walked sequentially.
static __device__ __noinline__ double lpg_logistic(const DevModel& M, const double* q, double* g, int jac, int lane) {
  const int D = M.K;  // predictors
  double alpha = q[0];
  double b[8], acc[8];
  const int per = (D + 31) / 32;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    int d = lane + 32 * i;
    b[i] = (i < per && d < D) ? q[1 + d] : 0.0;
    acc[i] = 0.0;
  }
  double lp = 0, ga = 0;
  for (int n = 0; n < M.N; ++n) {
    const double* x = M.X + (size_t)n * D;
    double part = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      int d = lane + 32 * i;
      if (i < per && d < D) part += x[d] * b[i];
    }
    double eta = alpha + wsum(part);
    int y = M.yi[n];
    lp += y * eta - log1p_exp(eta);
    double r = y - inv_logit(eta);
    ga += r;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      int d = lane + 32 * i;
      if (i < per && d < D) acc[i] += r * x[d];
    }
  }
  double pri = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    int d = lane + 32 * i;
    if (i < per && d < D) {
      pri += -0.5 * b[i] * b[i];
      g[1 + d] = acc[i] - b[i];
    }
  }
  lp += wsum(pri) - 0.5 * (alpha / 2.5) * (alpha / 2.5);
  if (lane == 0) g[0] = ga - alpha / 6.25;
  return lp;
}

// ---- varint: [alpha_1..J, beta_1..K, log sigma_y, log tau]; rows sorted by group.
// Members of a posterior set order the parameters [beta, log sigma_y, log tau,
// alpha] (alpha_last) and may evaluate the rows in FP32 (fp32).  The
// per-group scalar terms (alpha prior, its gradient) are spread over the
// lanes instead of being repeated by every lane.
// Rows are streamed independently of group boundaries: each lane takes rows
// lane, lane + 32, ..., four at a time with all their loads issued together;
// the residual sums per group (rows are sorted by group, so a warp's 32 rows
// span a few groups) are segmented warp reductions whose segment-end lane
// adds its total into g_al.  Row sums of squares and coefficient gradients
// are FP32 (T) per lane, added to FP64 every VR rows.
constexpr int VU = 4;   // rows per lane in flight
constexpr int VR = 32;  // rows per lane between FP64 flushes
template <class T>
__device__ __forceinline__ double varint_likelihood(const DevModel& M, const double* al, const double* bb,
                                                    double isy, double* g_al, double* gb, int lane) {
  const int J = M.J, K = M.K, N = M.N;
  T b[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) b[k] = (T)(k < K ? bb[k] : 0.0);
  const T tisy = (T)isy;
  for (int j = lane; j < J; j += 32) g_al[j] = 0.0;
  __syncwarp();
  double ss = 0;
  T s2 = 0, gk[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) gk[k] = 0;
  int since = 0;
  for (int base = 0; base < N; base += 32 * VU) {
    T x[VU][16], yv[VU];
    int grp[VU];
#pragma unroll
    for (int u = 0; u < VU; ++u) {
      const int n = base + 32 * u + lane;
      const bool ok = n < N;
      grp[u] = ok ? M.group[n] - 1 : 0x7fffffff;
      yv[u] = ok ? (T)M.yr[n] : (T)0;
      if constexpr (sizeof(T) == 4) {
        const float* xr = M.Xf + (size_t)(ok ? n : 0) * K;
#pragma unroll
        for (int k = 0; k < 16; ++k) x[u][k] = (ok && k < K) ? xr[k] : 0.f;
      } else {
        const double* xr = M.X + (size_t)(ok ? n : 0) * K;
#pragma unroll
        for (int k = 0; k < 16; ++k) x[u][k] = (ok && k < K) ? xr[k] : 0.0;
      }
    }
#pragma unroll
    for (int u = 0; u < VU; ++u) {
      const bool ok = grp[u] != 0x7fffffff;
      T mu = ok ? (T)al[grp[u]] : (T)0;
#pragma unroll
      for (int k = 0; k < 16; ++k)
        if (k < K) mu += x[u][k] * b[k];
      const T e = ok ? (yv[u] - mu) * tisy : (T)0;
      s2 += e * e;
      T r = e * tisy;
#pragma unroll
      for (int k = 0; k < 16; ++k)
        if (k < K) gk[k] += r * x[u][k];
      // segmented inclusive sum of r over lanes with the same group (keys ascend with the lane)
      const int key = grp[u];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const T rv = __shfl_up_sync(GN_FULL, r, o);
        const int kv = __shfl_up_sync(GN_FULL, key, o);
        if (lane >= o && kv == key) r += rv;
      }
      const int next = __shfl_down_sync(GN_FULL, key, 1);
      if (ok && (lane == 31 || next != key)) g_al[key] += (double)r;
      __syncwarp();
    }
    since += VU;
    if (since >= VR || base + 32 * VU >= N) {
      ss += (double)s2;
      s2 = 0;
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        gb[k] += (double)gk[k];
        gk[k] = 0;
      }
      since = 0;
    }
  }
  return ss;
}

static __device__ __noinline__ double lpg_varint(const DevModel& M, const double* q, double* g, int jac, int lane) {
  const int J = M.J, K = M.K;
  const int ib = M.alpha_last ? 0 : J, ia = M.alpha_last ? K + 2 : 0, is = M.alpha_last ? K : J + K;
  const double* al = q + ia;
  const double* be = q + ib;
  double ls = q[is], lt = q[is + 1];
  double sy = exp(ls), tau = exp(lt), isy = 1.0 / sy, itau = 1.0 / tau;
  double bb[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) bb[k] = k < K ? be[k] : 0.0;
  double gb[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) gb[k] = 0.0;
  // likelihood: residual sums per group into g[ia + j], shared coefficients into gb
  double ss = M.fp32 ? varint_likelihood<float>(M, al, bb, isy, g + ia, gb, lane)
                     : varint_likelihood<double>(M, al, bb, isy, g + ia, gb, lane);
  __syncwarp();
  // alpha_j ~ normal(0, tau), lane-parallel over groups
  double lpa = 0, glt = 0;
  for (int j = lane; j < J; j += 32) {
    const double z = al[j] * itau;
    g[ia + j] -= z * itau;
    lpa += -lt - 0.5 * z * z;
    glt += -1.0 + z * z;
  }
  lpa = wsum(lpa);
  glt = wsum(glt);
  ss = wsum(ss);
  double pb = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    if (k < K) {
      double t = wsum(gb[k]);
      if (lane == 0) g[ib + k] = t - bb[k];
      pb += -0.5 * bb[k] * bb[k];
    }
  }
  const double N = (double)M.N;
  double lp = lpa + pb - 0.5 * sy * sy - 0.5 * tau * tau - N * ls - 0.5 * ss;
  double gls = -sy * sy - N + ss;
  glt += -tau * tau;
  if (jac) {
    lp += ls + lt;
    gls += 1.0;
    glt += 1.0;
  }
  if (lane == 0) {
    g[is] = gls;
    g[is + 1] = glt;
  }
  return lp;
}

// ---- horseshoe logistic (warp version): [beta0, z_1..D, log tau, log lambda_1..D, log caux]
static __device__ __noinline__ double lpg_horseshoe(const DevModel& M, const double* q, double* g, int jac, int lane) {
  const int D = M.K;
  double b0 = q[0], lt = q[D + 1], tau = exp(lt), lc = q[2 * D + 2], caux = exp(lc);
  const double nu = M.slab_df, ssl = M.slab_scale, sg = M.scale_global;
  double c2 = ssl * ssl * caux;
  // beta held in global scratch g[] temporarily is unsafe (g is output); recompute per row block
  // lanes own coefficient d = lane + 32 i
  const int per = (D + 31) / 32;
  double beta[32], acc[32];
  for (int i = 0; i < per; ++i) {
    int d = lane + 32 * i;
    if (d < D) {
      double lam = exp(q[D + 2 + d]);
      double l2 = lam * lam;
      double lamt = sqrt(c2 * l2 / (c2 + tau * tau * l2));
      beta[i] = q[1 + d] * lamt * tau;
    } else {
      beta[i] = 0;
    }
    acc[i] = 0;
  }
  double lp = 0, gb0 = 0;
  for (int n = 0; n < M.N; ++n) {
    const double* x = M.X + (size_t)n * D;
    double part = 0;
    for (int i = 0; i < per; ++i) {
      int d = lane + 32 * i;
      if (d < D) part += x[d] * beta[i];
    }
    double eta = b0 + wsum(part);
    int y = M.yi[n];
    lp += y * eta - log1p_exp(eta);
    double r = y - inv_logit(eta);
    gb0 += r;
    for (int i = 0; i < per; ++i) {
      int d = lane + 32 * i;
      if (d < D) acc[i] += r * x[d];
    }
  }
  double pri = 0, glt = 0, glc = 0;
  for (int i = 0; i < per; ++i) {
    int d = lane + 32 * i;
    if (d < D) {
      double z = q[1 + d];
      double lam = exp(q[D + 2 + d]);
      double l2 = lam * lam;
      double den = c2 + tau * tau * l2;
      double a = c2 / den, bt = tau * tau * l2 / den;
      double lamt = sqrt(c2 * l2 / den);
      double gbd = acc[i] * beta[i];
      pri += -0.5 * z * z - log1p(l2) + (jac ? q[D + 2 + d] : 0.0);
      g[1 + d] = acc[i] * lamt * tau - z;
      g[D + 2 + d] = gbd * a - 2.0 * l2 / (1.0 + l2) + (jac ? 1.0 : 0.0);
      glt += gbd * (1.0 - bt);
      glc += gbd * 0.5 * bt;
    }
  }
  pri = wsum(pri);
  glt = wsum(glt);
  glc = wsum(glc);
  double ts = tau / sg;
  lp += pri - 0.5 * (b0 / 2.5) * (b0 / 2.5) - log1p(ts * ts) + (-0.5 * nu - 1.0) * lc - 0.5 * nu / caux;
  glt += -2.0 * ts * ts / (1.0 + ts * ts);
  glc += (-0.5 * nu - 1.0) + 0.5 * nu / caux;
  if (jac) {
    lp += lt + lc;
    glt += 1.0;
    glc += 1.0;
  }
  if (lane == 0) {
    g[0] = gb0 - b0 / 6.25;
    g[D + 1] = glt;
    g[2 * D + 2] = glc;
  }
  return lp;
}

__device__ __forceinline__ double warp_log_prob_grad(const DevModel& M, const double* q, double* g,
                                                     int jac, int lane) {
  switch (M.kind) {
    case MK_BERNOULLI: return lpg_bernoulli(M, q, g, jac, lane);
    case MK_NORMAL: return lpg_normal(M, q, g, jac, lane);
    case MK_LOGISTIC: return lpg_logistic(M, q, g, jac, lane);
    case MK_HIER: return lpg_hier(M, q, g, jac, lane);
    case MK_FUNNEL: return lpg_funnel(M, q, g, jac, lane);
    case MK_VARINT: return lpg_varint(M, q, g, jac, lane);
    case MK_HORSESHOE: return lpg_horseshoe(M, q, g, jac, lane);
  }
  return __longlong_as_double(0x7ff8000000000000ll);
}

// the same for a model kind known at compile time (kernels instantiated per
// kind carry only that model's code)
template <int KIND>
__device__ __forceinline__ double warp_lpg_k(const DevModel& M, const double* q, double* g, int jac, int lane) {
  if constexpr (KIND == MK_BERNOULLI) return lpg_bernoulli(M, q, g, jac, lane);
  else if constexpr (KIND == MK_NORMAL) return lpg_normal(M, q, g, jac, lane);
  else if constexpr (KIND == MK_LOGISTIC) return lpg_logistic(M, q, g, jac, lane);
  else if constexpr (KIND == MK_HIER) return lpg_hier(M, q, g, jac, lane);
  else if constexpr (KIND == MK_FUNNEL) return lpg_funnel(M, q, g, jac, lane);
  else if constexpr (KIND == MK_VARINT) return lpg_varint(M, q, g, jac, lane);
  else return lpg_horseshoe(M, q, g, jac, lane);
}

// the model a chain (or point) c of C evaluates: itself, or its posterior-set member
__device__ __forceinline__ const DevModel& chain_model(const DevModel& M, int c, int C) {
  return M.members ? M.members[c / (C / M.n_members)] : M;
}

// write_array: unconstrained q -> constrained output columns (team-parallel:
// thread `lane` of TW)
template <int TW = 32>
__device__ __forceinline__ void warp_write_array(const DevModel& M, const double* q, double* out,
                                                 int lane) {
  switch (M.kind) {
    case MK_BERNOULLI:
      if (lane == 0) out[0] = inv_logit(q[0]);
      return;
    case MK_NORMAL:
    case MK_LOGISTIC:
    case MK_FUNNEL:
      for (int i = lane; i < M.D; i += TW) out[i] = q[i];
      return;
    case MK_HIER:
      for (int i = lane; i < M.D; i += TW) out[i] = (i == M.J + 1) ? exp(q[i]) : q[i];
      return;
    case MK_VARINT: {
      const int is = M.alpha_last ? M.K : M.J + M.K;
      for (int i = lane; i < M.D; i += TW) out[i] = (i == is || i == is + 1) ? exp(q[i]) : q[i];
      return;
    }
    case MK_HORSESHOE: {
      const int D = M.K;
      double tau = exp(q[D + 1]), caux = exp(q[2 * D + 2]);
      double c2 = M.slab_scale * M.slab_scale * caux;
      for (int i = lane; i < 2 * D + 3; i += TW) out[i] = (i <= D) ? q[i] : exp(q[i]);
      for (int d = lane; d < D; d += TW) {
        double lam = exp(q[D + 2 + d]);
        double l2 = lam * lam;
        double lamt = sqrt(c2 * l2 / (c2 + tau * tau * l2));
        out[2 * D + 3 + d] = q[1 + d] * lamt * tau;
      }
      return;
    }
  }
}

}  // namespace gnuts

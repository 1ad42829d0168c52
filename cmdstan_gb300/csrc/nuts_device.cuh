// Per-chain NUTS state machine on the device.
//
// Replaces stan::mcmc::base_nuts::transition / build_tree, expl_leapfrog,
// the diag_e / dense_e / unit_e metrics, stepsize_adaptation and the
// windowed var / covar adaptation that the hmc_nuts_* services run
// (called from src/cmdstan/command.hpp:609-632 and 657-688).
//
// The recursion of build_tree becomes an explicit stack: a doubling of depth
// d visits leaves k = 0 .. 2^d-1 in order; after leaf k the pending left
// subtrees at heights h with bit h of k set are merged bottom-up (post-order,
// as the recursion does), otherwise the current subtree is parked at its
// height.  Subtree summaries live in a per-chain pool of records
// {p_beg, p#_beg, p_end, p#_end, rho, proposal q, proposal grad} addressed by
// index, so merges and pushes move indices, not vectors.
//
// A team of TW threads advances one chain -- one warp (TW = 32), or a CTA
// (TW = 256) for wide chains, whose per-element work would otherwise run 63
// elements deep per lane on one warp scheduler; thread l owns vector elements
// l, l + TW, ...  Every thread carries the same scalar state (team-uniform
// control flow); team sums hand every thread the same bits.
// advance() runs the machine until the chain needs the gradient at W.q (it
// returns true) or the chain is finished (false).  The gradient is written
// into W.g / W_lp by the caller: inline (fused kernel) or by a batched
// gradient kernel (round mode).
#pragma once
#include "device_models.cuh"
#include "philox.cuh"

namespace gnuts {

enum Phase : int { PH_INIT = 0, PH_IS_FIRST = 1, PH_IS_LOOP = 2, PH_LEAF = 3, PH_DONE = 4, PH_ERROR = 5 };
enum ChainErr : int { CE_OK = 0, CE_INIT = 1, CE_IMPROPER = 2, CE_NO_STEPSIZE = 3, CE_METRIC = 4, CE_NOT_PD = 5 };

constexpr int MAXREC = 18;  // max_depth <= 16

struct Scal {
  int phase, err, iter, row;
  int depth, n_leapfrog, divergent, dir;
  int leaf, cur;
  unsigned free_mask;
  int is_dir, is_ctx, init_attempts, adapt_done, pad0;
  double nom_eps, eps, H0, lsw, sum_metro;
  double W_lp, F_lp, B_lp, S_lp, S_h;
  double is_H0;
  double da_mu, da_counter, da_sbar, da_xbar;
  unsigned w_nw, w_ib, w_tb, w_bw, w_counter, w_size, w_next, pad1;
  double wf_n;
  unsigned long long rng_n, irng_n;
  long long n_grad, n_lf_total;
  unsigned long long t_start, t_warm, t_end;
  // pending left subtree per height: 5-bit record indices (31 = none),
  // heights 0..11 in stk_lo, 12..17 in stk_hi
  unsigned long long stk_lo, stk_hi;
};

struct Params {
  int C, D, ld, ncon, ncol, R;
  int metric, adapt;
  int num_warmup, num_samples, thin, save_warmup;
  double stepsize, jitter;
  int max_depth;
  double delta, gamma, kappa, t0;
  unsigned init_buffer, term_buffer, window;
  unsigned seed, id_base;
  double init_radius;
  int has_init, replay, n_saved, grad_budget;
  int cache;          // chain vectors cached in shared memory during a launch
  int cache_stride;   // doubles of shared memory per warp when cached
  int diag;           // diagnostic rows wanted: track the selected point's momentum
  int nrv;            // vectors per subtree record: 7, or 8 with diag (proposal momentum)
  int dense32;        // dense metric of a team-mode chain on the mixed path: metric
                      // product, momentum draw and Welford covariance in FP32
};

// largest D of the FP32 dense path (its vectors are staged in shared memory)
constexpr int DENSE32_MAXD = 2048;

// vectors cached per chain (diag / unit metric also caches minv, wm, wm2)
constexpr int NCACHE_VEC = 17;
constexpr int NCACHE_VEC_DIAG = 20;
// elements per lane whose loads are issued together: VCH in the record
// loops (merge, finish_doubling: nine or ten vectors), Chain::VCW in the
// loops over at most four vectors (leapfrog, leaf record, dot, metric
// product, copies)
constexpr int VCH = 4;
constexpr int VC1 = 4;  // elements per lane of the one-pass leaf step (D <= 128)

struct Bufs {
  double *Wq, *Wp, *Wg, *Fq, *Fp, *Fg, *Bq, *Bp, *Bg, *Sq, *Sg;
  double *Tpb, *Tsb, *Tpe, *Tse, *Trho;
  double* rec;   // [C][R][nrv][ld]
  double* recs;  // [C][R][3]: log-sum-weight, proposal lp, proposal energy of each record
  double* minv;  // diag/unit [C][ld]; dense [C][D][ld]
  double* chol;  // dense: transposed Cholesky factor Lt[k][i] = L[i][k], [C][D][ld]
  double *wm, *wm2, *tmp;
  double* draws;       // [C][n_saved][ncol]
  double* out_eps;     // [C]
  double* out_minv;    // [C][D] or [C][D*D]
  const double* init_q;  // [C][D] (has_init)
  const double* p0;      // [C][D] (replay)
  const double* init_eps;  // [C] per-chain initial step size (null: P.stepsize)
  double* zdraws;        // [C][n_saved][D]: sampler-space draws (flow runs; write_array happens later)
  double* Sp;            // [C][ld] momentum of the selected point (diag)
  double* diag_draws;    // [C][n_saved][7 + 3D]: sampler columns, q, p, gradient (diag)
  float *minv32, *chol32;          // dense32: FP32 copies of minv and chol [C][D][ld]
  float *wm2_32, *wm2_32lo;         // dense32: Welford sums as float-float pairs (hi, lo) [C][D][ld]
  float* wpend;   // dense32: a pending Welford sample per chain [C][4][ld]: b hi, b lo, a hi, a lo
  int* wlist;     // dense32: [0] pending count, [1] finished-CTA count, [2 + k] chain ids
  Scal* sc;
  int* done_count;
};

// record vector slots
enum { RV_PB = 0, RV_SB = 1, RV_PE = 2, RV_SE = 3, RV_RHO = 4, RV_Q = 5, RV_G = 6, RV_P = 7 };

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ double lse(double a, double b) {
  const double NEG_INF = -__longlong_as_double(0x7ff0000000000000ll);
  if (a == NEG_INF) return b;
  if (b == NEG_INF) return a;
  double m = a > b ? a : b;
  return m + log1p(exp(-fabs(a - b)));
}

// MET >= 0 fixes the metric at compile time (0 diag_e, 1 dense_e, 2 unit_e):
// a kernel instantiated per metric carries only that metric's code on its
// hot path; MET = -1 reads it from the run's parameters.
// float-float accumulation (hi, lo) += (a0 + a1) (b0 + b1): the product of
// the leading parts split exactly (two-product), the cross terms added to its
// error, the sum formed with a two-sum and renormalised
__device__ __forceinline__ void ff_axpy(float& hi_io, float& lo_io, float a0, float a1, float b0, float b1) {
  const float pr = a0 * b0;
  const float pe = fmaf(a0, b1, fmaf(a1, b0, fmaf(a0, b0, -pr)));
  const float hi = hi_io;
  const float sm = hi + pr;
  const float bv = sm - hi;
  const float t = ((hi - (sm - bv)) + (pr - bv)) + (lo_io + pe);
  const float nh = sm + t;
  hi_io = nh;
  lo_io = t - (nh - sm);
}

template <int MET = -1, int TW = 32>
struct Chain {
  // chunk of the loops over at most four vectors: 4 elements per lane for a
  // warp (D up to about 128: less masked FP64 work per chunk), 8 for a team
  // (a wide chain's 16 elements per thread in two chunks).  Each lane visits
  // its elements in increasing order either way, so sums do not change.
  static constexpr int VCW = TW == 32 ? 4 : 8;
  const Params& P;
  const Bufs& B;
  const DevModel& M;
  Scal& s;
  int c, lane, D;
  uint32_t chain_id;
  double *Wq, *Wp, *Wg, *Fq, *Fp, *Fg, *Bq, *Bp, *Bg, *Sq, *Sg, *Tpb, *Tsb, *Tpe, *Tse, *Trho;
  double *minv, *chol, *wm, *wm2, *tmp;
  double* Sp;   // momentum of the selected point (diagnostic rows only)
  float *m32 = nullptr, *l32 = nullptr, *w32 = nullptr, *w32lo = nullptr;  // dense32 matrices of this chain
  double* rsc;  // this chain's record scalars [R][3]
  double* cache_base = nullptr;

  __device__ Chain(const Params& p, const Bufs& b, const DevModel& m, Scal& sc, int ci, int ln)
      : P(p), B(b), M(m), s(sc), c(ci), lane(ln), D(m.D) {
    rsc = b.recs + (size_t)ci * p.R * 3;
    chain_id = p.id_base + (uint32_t)ci;
    size_t o = (size_t)ci * p.ld;
    Wq = b.Wq + o; Wp = b.Wp + o; Wg = b.Wg + o;
    Fq = b.Fq + o; Fp = b.Fp + o; Fg = b.Fg + o;
    Bq = b.Bq + o; Bp = b.Bp + o; Bg = b.Bg + o;
    Sq = b.Sq + o; Sg = b.Sg + o;
    Tpb = b.Tpb + o; Tsb = b.Tsb + o; Tpe = b.Tpe + o; Tse = b.Tse + o; Trho = b.Trho + o;
    tmp = b.tmp + o;
    size_t mo = p.metric == 1 ? (size_t)ci * p.D * p.ld : o;
    minv = b.minv + mo;
    chol = p.metric == 1 ? b.chol + mo : nullptr;
    wm = b.wm + o;
    wm2 = b.wm2 + mo;
    Sp = b.Sp ? b.Sp + o : nullptr;
    if (TW > 32 && p.dense32) {
      m32 = b.minv32 + mo;
      l32 = b.chol32 + mo;
      w32 = b.wm2_32 + mo;
      w32lo = b.wm2_32lo + mo;
    }
  }
  // only the round-mode team kernel of the dense metric (MET = 1) carries this code
  __device__ __forceinline__ bool dense32() const { return TW > 32 && MET == 1 && m32 != nullptr; }
  // the team's FP32 staging vectors (shared memory, four of DENSE32_MAXD;
  // the dense32 steps that use them -- metric product, momentum solve,
  // Welford update -- never overlap)
  static __device__ __forceinline__ float* fbuf() {
    __shared__ float b[4 * DENSE32_MAXD];
    return b;
  }
  __device__ __forceinline__ int metric() const { return MET >= 0 ? MET : P.metric; }
  __device__ double* rec(int r, int v) const {
    return B.rec + (((size_t)c * P.R + r) * P.nrv + v) * P.ld;
  }
  // record scalars: every lane writes the same value; a full-warp shuffle or
  // __syncwarp separates reads from later writes of the same record
  __device__ double& rlsw(int r) const { return rsc[r * 3 + 0]; }
  __device__ double& rlp(int r) const { return rsc[r * 3 + 1]; }
  __device__ double& rh(int r) const { return rsc[r * 3 + 2]; }
  __device__ int stack_get(int h) const {
    const unsigned long long w = h < 12 ? s.stk_lo : s.stk_hi;
    return (int)((w >> (5 * (h < 12 ? h : h - 12))) & 31ull);
  }
  __device__ void stack_set(int h, int v) {
    const int sh = 5 * (h < 12 ? h : h - 12);
    const unsigned long long m = ~(31ull << sh), x = (unsigned long long)(v & 31) << sh;
    if (h < 12) s.stk_lo = (s.stk_lo & m) | x;
    else s.stk_hi = (s.stk_hi & m) | x;
  }

  // ---------------- shared-memory cache of the chain's vectors ----------------
  // One launch loads the chain's working vectors into this warp's slice of
  // shared memory (independent loads, all in flight at once) and writes them
  // back at exit, so the state machine's dependent accesses stay on chip.
  __device__ int cached_vectors() const { return metric() == 1 ? NCACHE_VEC : NCACHE_VEC_DIAG; }
  template <class F>
  __device__ void for_each_cached(F f) {
    double** v[NCACHE_VEC_DIAG] = {&Wq, &Wp, &Wg, &Fq, &Fp, &Fg, &Bq, &Bp, &Bg, &Sq,
                                   &Sg, &Tpb, &Tsb, &Tpe, &Tse, &Trho, &tmp, &minv, &wm, &wm2};
    const int n = cached_vectors();
#pragma unroll
    for (int i = 0; i < NCACHE_VEC_DIAG; ++i)
      if (i < n) f(i, v[i]);
  }
  // global -> shared copies go through cp.async: no register round trip, all
  // of them in flight at once, one wait at the end
  static __device__ __forceinline__ void cp_async8(double* smem_dst, const double* gmem_src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(smem_dst)),
                 "l"(gmem_src)
                 : "memory");
  }
  __device__ void cache_attach(double* base) {
    cache_base = base;
    for_each_cached([&](int i, double** p) {
      const double* gsrc = *p;
      double* sm = base + (size_t)i * P.ld;
      for (int d = lane; d < D; d += TW) cp_async8(sm + d, gsrc + d);
      *p = sm;
    });
    double* sr = base + (size_t)cached_vectors() * P.ld;
    for (int i = lane; i < P.R * 3; i += TW) cp_async8(sr + i, rsc + i);
    rsc = sr;
    asm volatile("cp.async.wait_all;" ::: "memory");
    tsync<TW>();
  }
  __device__ void cache_detach() {
    tsync<TW>();
    const size_t o = (size_t)c * P.ld;
    double* g[NCACHE_VEC_DIAG] = {B.Wq + o, B.Wp + o, B.Wg + o, B.Fq + o, B.Fp + o, B.Fg + o, B.Bq + o,
                                  B.Bp + o, B.Bg + o, B.Sq + o, B.Sg + o, B.Tpb + o, B.Tsb + o, B.Tpe + o,
                                  B.Tse + o, B.Trho + o, B.tmp + o, B.minv + o, B.wm + o, B.wm2 + o};
    for_each_cached([&](int i, double** p) {
      for (int d = lane; d < D; d += TW) g[i][d] = (*p)[d];
    });
    double* gr = B.recs + (size_t)c * P.R * 3;
    for (int i = lane; i < P.R * 3; i += TW) gr[i] = rsc[i];
  }

  // ---------------- vector helpers ----------------
  // chunks of VCW elements per lane: every load of a chunk is issued before
  // its stores, so a copy costs one memory round trip per TW VCW elements
  __device__ void copy(double* dst, const double* src) const {
    for (int base = 0; base < D; base += TW * VCW) {
      double v[VCW];
#pragma unroll
      for (int j = 0; j < VCW; ++j) {
        const int d = base + lane + TW * j;
        v[j] = d < D ? src[d] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < VCW; ++j) {
        const int d = base + lane + TW * j;
        if (d < D) dst[d] = v[j];
      }
    }
  }
  __device__ void copy2(double* d1, const double* s1, double* d2, const double* s2) const {
    for (int base = 0; base < D; base += TW * VCW) {
      double v[VCW], w[VCW];
#pragma unroll
      for (int j = 0; j < VCW; ++j) {
        const int d = base + lane + TW * j;
        v[j] = d < D ? s1[d] : 0.0;
        w[j] = d < D ? s2[d] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < VCW; ++j) {
        const int d = base + lane + TW * j;
        if (d < D) {
          d1[d] = v[j];
          d2[d] = w[j];
        }
      }
    }
  }
  __device__ void copy3(double* d1, const double* s1, double* d2, const double* s2, double* d3,
                        const double* s3) const {
    for (int base = 0; base < D; base += TW * VCW) {
      double u[VCW], v[VCW], w[VCW];
#pragma unroll
      for (int j = 0; j < VCW; ++j) {
        const int d = base + lane + TW * j;
        u[j] = d < D ? s1[d] : 0.0;
        v[j] = d < D ? s2[d] : 0.0;
        w[j] = d < D ? s3[d] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < VCW; ++j) {
        const int d = base + lane + TW * j;
        if (d < D) {
          d1[d] = u[j];
          d2[d] = v[j];
          d3[d] = w[j];
        }
      }
    }
  }
  // The element loops below run in chunks of VCW elements per lane with every
  // load of a chunk issued before its arithmetic and stores: the vectors live
  // in global (or shared) memory behind pointers the compiler must assume may
  // alias, so a plain loop makes each element a full memory round trip (63 of
  // them per vector at D = 2003).  Each element's arithmetic and each lane's
  // summation order are those of the plain loop.
  __device__ double dot(const double* a, const double* b) const {
    double t = 0;
    for (int base = 0; base < D; base += TW * VCW) {
      double va[VCW], vb[VCW];
#pragma unroll
      for (int j = 0; j < VCW; ++j) {
        const int d = base + lane + TW * j;
        va[j] = d < D ? a[d] : 0.0;
        vb[j] = d < D ? b[d] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < VCW; ++j)
        if (base + lane + TW * j < D) t += va[j] * vb[j];
    }
    return tsum<TW>(t);
  }
  // out = minv * p  (p must be visible to the whole warp for dense)
  __device__ void dtau(double* out, const double* p) const {
    if (metric() != 1) {
      for (int base = 0; base < D; base += TW * VCW) {
        double vm[VCW], vp[VCW];
#pragma unroll
        for (int j = 0; j < VCW; ++j) {
          const int d = base + lane + TW * j;
          vp[j] = d < D ? p[d] : 0.0;
          vm[j] = d < D && metric() == 0 ? minv[d] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < VCW; ++j) {
          const int d = base + lane + TW * j;
          if (d < D) out[d] = metric() == 0 ? vm[j] * vp[j] : vp[j];
        }
      }
    } else if (dense32()) {
      dtau32(out, p);
    } else {
      tsync<TW>();
      for (int d = lane; d < D; d += TW) {
        double t = 0;
        for (int j = 0; j < D; ++j) t += minv[(size_t)j * P.ld + d] * p[j];
        out[d] = t;
      }
    }
  }
  // dense32 metric product: p staged in FP32 in shared memory; thread l
  // forms outputs 4l .. 4l + 3 of each group of 4 TW (four groups per pass)
  // from 16-byte loads of rows of the symmetric FP32 minv (ld is a multiple
  // of 4, so the loads are aligned and stay inside the row's padding),
  // accumulating in FP32 in row order
  __device__ void dtau32(double* out, const double* p) const {
    float* ps = fbuf();
    tsync<TW>();
    for (int d = lane; d < D; d += TW) ps[d] = (float)p[d];
    tsync<TW>();
    constexpr int NG = 4;
    for (int d0 = 0; d0 < D; d0 += 4 * TW * NG) {
      float4 acc[NG];
#pragma unroll
      for (int g = 0; g < NG; ++g) acc[g] = make_float4(0.f, 0.f, 0.f, 0.f);
      const int db = d0 + 4 * lane;
#pragma unroll 2
      for (int j = 0; j < D; ++j) {
        const float pj = ps[j];
        const float4* row = reinterpret_cast<const float4*>(m32 + (size_t)j * P.ld + db);
#pragma unroll
        for (int g = 0; g < NG; ++g)
          if (db + 4 * TW * g < D) {
            const float4 m = row[TW * g];
            acc[g].x = fmaf(m.x, pj, acc[g].x);
            acc[g].y = fmaf(m.y, pj, acc[g].y);
            acc[g].z = fmaf(m.z, pj, acc[g].z);
            acc[g].w = fmaf(m.w, pj, acc[g].w);
          }
      }
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const int d = db + 4 * TW * g;
        const float v[4] = {acc[g].x, acc[g].y, acc[g].z, acc[g].w};
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (d + e < D) out[d + e] = (double)v[e];
      }
    }
    tsync<TW>();
  }
  // kinetic energy 0.5 p.(minv p), using a precomputed ps = minv p
  __device__ double kinetic(const double* p, const double* ps) const { return 0.5 * dot(p, ps); }

  __device__ void sample_p(double* p) {
    const uint64_t n0 = s.rng_n;
    if (dense32()) {
      for (int d = lane; d < D; d += TW) tmp[d] = rng_normal(P.seed, chain_id, 0u, n0 + (uint64_t)(d >> 1), d & 1);
      solve_lt32(p);
    } else if (metric() == 1) {
      for (int d = lane; d < D; d += TW) tmp[d] = rng_normal(P.seed, chain_id, 0u, n0 + (uint64_t)(d >> 1), d & 1);
      tsync<TW>();
      // solve Lt p = z, back substitution over rows of Lt (Lt[i][k] = L[k][i])
      for (int i = D - 1; i >= 0; --i) {
        const double* row = chol + (size_t)i * P.ld;
        double t = 0;
        for (int k = i + 1 + lane; k < D; k += TW) t += row[k] * p[k];
        t = tsum<TW>(t);
        double v = (tmp[i] - t) / row[i];
        if (lane == i % TW) p[i] = v;
        tsync<TW>();
      }
    } else {
      for (int d = lane; d < D; d += TW) {
        double z = rng_normal(P.seed, chain_id, 0u, n0 + (uint64_t)(d >> 1), d & 1);
        p[d] = metric() == 0 ? z / sqrt(minv[d]) : z;
      }
    }
    s.rng_n = n0 + (uint64_t)((D + 1) / 2);
    tsync<TW>();
  }
  __device__ double uniform() { return rng_uniform(P.seed, chain_id, 0u, s.rng_n++); }

  // dense32 momentum: solve Lt p = z (z in tmp) in FP32, 32 rows per block
  // from the bottom.  For block [i0, i0 + 32) the team first forms each row's
  // sum over the solved entries k >= i0 + 32 (thread t takes k = i0 + 32 + t,
  // + TW, ...; a warp reduce-scatter leaves row i0 + l's sum with lane l, and
  // the warps' sums are added in warp order), then warp 0 solves the 32 x 32
  // triangle with shuffles.
  __device__ void solve_lt32(double* p) {
    float* ps = fbuf();
    __shared__ float red[TW / 32][32];
    const int wid = lane >> 5, ln = lane & 31;
    tsync<TW>();
    for (int i1 = D; i1 > 0; i1 -= 32) {
      const int i0 = max(0, i1 - 32), nb = i1 - i0;
      float acc[32];
#pragma unroll
      for (int r = 0; r < 32; ++r) acc[r] = 0.f;
      for (int k = i1 + lane; k < D; k += TW) {
        const float pk = ps[k];
#pragma unroll
        for (int r = 0; r < 32; ++r)
          if (r < nb) acc[r] = fmaf(l32[(size_t)(i0 + r) * P.ld + k], pk, acc[r]);
      }
      // reduce-scatter over the warp: after the five steps lane l holds row l
#pragma unroll
      for (int h = 16; h >= 1; h >>= 1) {
        const bool upper = (ln & h) != 0;
#pragma unroll
        for (int r = 0; r < h; ++r) {
          const float send = upper ? acc[r] : acc[r + h];
          const float keep = upper ? acc[r + h] : acc[r];
          acc[r] = keep + __shfl_xor_sync(0xffffffffu, send, h);
        }
      }
      if constexpr (TW > 32) {
        red[wid][ln] = acc[0];
        tsync<TW>();
      }
      if (wid == 0) {
        float rsum = 0.f;
        if constexpr (TW > 32) {
#pragma unroll
          for (int w = 0; w < TW / 32; ++w) rsum += red[w][ln];
        } else {
          rsum = acc[0];
        }
        // row i0 + ln: (z - rsum - sum over the block's later rows) / diagonal
        float v = ln < nb ? (float)tmp[i0 + ln] - rsum : 0.f;
        const float* row = l32 + (size_t)(i0 + (ln < nb ? ln : 0)) * P.ld;
        for (int r = nb - 1; r >= 0; --r) {
          float pr = 0.f;
          if (ln == r) pr = v / row[i0 + r];
          pr = __shfl_sync(0xffffffffu, pr, r);
          if (ln < r) v = fmaf(-row[i0 + r], pr, v);
          if (ln == r) {
            ps[i0 + r] = pr;
            p[i0 + r] = (double)pr;
          }
        }
      }
      tsync<TW>();
    }
  }

  // W.p += e/2 g ; W.q += e * minv W.p   (gradient at W.q then requested)
  __device__ void begin_leapfrog(double e) {
    if (metric() == 1) {
      for (int d = lane; d < D; d += TW) Wp[d] += 0.5 * e * Wg[d];
      dtau(tmp, Wp);
      for (int d = lane; d < D; d += TW) Wq[d] += e * tmp[d];
    } else {
      for (int base = 0; base < D; base += TW * VCW) {
        double vp[VCW], vg[VCW], vq[VCW], vm[VCW];
#pragma unroll
        for (int j = 0; j < VCW; ++j) {
          const int d = base + lane + TW * j;
          const bool ok = d < D;
          vp[j] = ok ? Wp[d] : 0.0;
          vg[j] = ok ? Wg[d] : 0.0;
          vq[j] = ok ? Wq[d] : 0.0;
          vm[j] = ok && metric() == 0 ? minv[d] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < VCW; ++j) {
          const int d = base + lane + TW * j;
          if (d < D) {
            const double pn = vp[j] + 0.5 * e * vg[j];
            Wp[d] = pn;
            Wq[d] = vq[j] + e * (metric() == 0 ? vm[j] * pn : pn);
          }
        }
      }
    }
    tsync<TW>();
  }
  __device__ void complete_leapfrog(double e) {
    for (int base = 0; base < D; base += TW * VCW) {
      double vp[VCW], vg[VCW];
#pragma unroll
      for (int j = 0; j < VCW; ++j) {
        const int d = base + lane + TW * j;
        vp[j] = d < D ? Wp[d] : 0.0;
        vg[j] = d < D ? Wg[d] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < VCW; ++j) {
        const int d = base + lane + TW * j;
        if (d < D) Wp[d] = vp[j] + 0.5 * e * vg[j];
      }
    }
    ++s.n_grad;
    tsync<TW>();
  }
  __device__ double energy_W(double* ps) {
    dtau(ps, Wp);
    return kinetic(Wp, ps) - s.W_lp;
  }
  __device__ void load_W_from(const double* q, const double* p, const double* g, double lp) {
    if (p) copy3(Wq, q, Wp, p, Wg, g);
    else copy2(Wq, q, Wg, g);
    s.W_lp = lp;
    tsync<TW>();
  }

  // ---------------- error / completion ----------------
  __device__ void fail(int code) {
    s.err = code;
    s.phase = PH_ERROR;
    s.t_end = globaltimer();
    if (lane == 0) atomicAdd(B.done_count, 1);
  }
  __device__ void finish() {
    s.phase = PH_DONE;
    s.t_end = globaltimer();
    if (lane == 0) atomicAdd(B.done_count, 1);
  }

  // ---------------- initialisation ----------------
  // draws a candidate into W.q (stream 1), gradient then requested
  __device__ void init_candidate() {
    if (P.has_init) {
      for (int d = lane; d < D; d += TW) Wq[d] = B.init_q[(size_t)c * P.D + d];
    } else {
      const uint64_t n0 = s.irng_n;
      for (int d = lane; d < D; d += TW)
        Wq[d] = P.init_radius * (2.0 * rng_uniform(P.seed, chain_id, 1u, n0 + (uint64_t)d) - 1.0);
      s.irng_n = n0 + (uint64_t)D;
    }
    ++s.init_attempts;
    s.phase = PH_INIT;
    tsync<TW>();
  }
  __device__ bool W_finite() const {
    bool ok = isfinite(s.W_lp);
    for (int d = lane; d < D; d += TW) ok = ok && isfinite(Wg[d]);
    return tall<TW>(ok);
  }

  // ---------------- step-size search ----------------
  // returns true if a gradient is requested
  __device__ bool begin_init_stepsize(int ctx) {
    s.is_ctx = ctx;
    if (s.nom_eps == 0 || s.nom_eps > 1e7 || isnan(s.nom_eps)) return after_init_stepsize();
    load_W_from(Sq, nullptr, Sg, s.S_lp);
    sample_p(Wp);
    s.is_H0 = energy_W(tmp);
    begin_leapfrog(s.nom_eps);
    s.phase = PH_IS_FIRST;
    return true;
  }
  __device__ bool after_init_stepsize() {
    if (s.is_ctx == 1) {
      s.da_mu = log(10.0 * s.nom_eps);
      s.da_counter = 0; s.da_sbar = 0; s.da_xbar = 0;
    }
    return begin_transition();
  }
  __device__ bool step_init_stepsize() {
    complete_leapfrog(s.nom_eps);
    double h = energy_W(tmp);
    if (isnan(h)) h = __longlong_as_double(0x7ff0000000000000ll);
    double dH = s.is_H0 - h;
    const double l08 = -0.22314355131420976;  // log(0.8)
    if (s.phase == PH_IS_FIRST) {
      s.is_dir = dH > l08 ? 1 : -1;
    } else {
      if (s.is_dir == 1 && !(dH > l08)) return after_init_stepsize();
      if (s.is_dir == -1 && !(dH < l08)) return after_init_stepsize();
      s.nom_eps = s.is_dir == 1 ? 2.0 * s.nom_eps : 0.5 * s.nom_eps;
      if (s.nom_eps > 1e7) { fail(CE_IMPROPER); return false; }
      if (s.nom_eps == 0) { fail(CE_NO_STEPSIZE); return false; }
    }
    load_W_from(Sq, nullptr, Sg, s.S_lp);
    sample_p(Wp);
    s.is_H0 = energy_W(tmp);
    begin_leapfrog(s.nom_eps);
    s.phase = PH_IS_LOOP;
    return true;
  }

  // ---------------- transition ----------------
  __device__ int alloc_rec() {
    int r = __ffs(s.free_mask) - 1;
    s.free_mask &= ~(1u << r);
    return r;
  }
  __device__ void free_rec(int r) { s.free_mask |= (1u << r); }

  __device__ bool begin_transition() {
    const int total = P.num_warmup + P.num_samples;
    if (s.iter >= total) { finish(); return false; }
    if (s.iter == P.num_warmup && !s.adapt_done) {
      s.adapt_done = 1;
      if (P.adapt) s.nom_eps = exp(s.da_xbar);  // complete_adaptation
      s.t_warm = globaltimer();
      if (lane == 0) B.out_eps[c] = s.nom_eps;
      const size_t msz = metric() == 1 ? (size_t)D * D : (size_t)P.D;
      if (metric() == 1) {
        for (int i = 0; i < D; ++i)
          for (int j = lane; j < D; j += TW) B.out_minv[(size_t)c * msz + (size_t)i * D + j] = minv[(size_t)i * P.ld + j];
      } else {
        for (int d = lane; d < D; d += TW) B.out_minv[(size_t)c * msz + d] = minv[d];
      }
    }
    s.eps = s.nom_eps;
    if (P.jitter > 0 && !P.replay) s.eps *= 1.0 + P.jitter * (2.0 * uniform() - 1.0);
    load_W_from(Sq, nullptr, Sg, s.S_lp);
    if (P.replay) {
      for (int d = lane; d < D; d += TW) Wp[d] = B.p0[(size_t)c * P.D + d];
      tsync<TW>();
    } else {
      sample_p(Wp);
    }
    dtau(Tsb, Wp);
    s.H0 = kinetic(Wp, Tsb) - s.W_lp;
    s.S_h = s.H0;
    for (int base = 0; base < D; base += TW * VCW) {
      double vp[VCW], vq[VCW], vg[VCW], vs[VCW];
#pragma unroll
      for (int j = 0; j < VCW; ++j) {
        const int d = base + lane + TW * j;
        const bool ok = d < D;
        vp[j] = ok ? Wp[d] : 0.0;
        vq[j] = ok ? Wq[d] : 0.0;
        vg[j] = ok ? Wg[d] : 0.0;
        vs[j] = ok ? Tsb[d] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < VCW; ++j) {
        const int d = base + lane + TW * j;
        if (d < D) {
          const double p = vp[j];
          Fq[d] = vq[j]; Fp[d] = p; Fg[d] = vg[j];
          Bq[d] = vq[j]; Bp[d] = p; Bg[d] = vg[j];
          Tpb[d] = p; Tpe[d] = p; Tse[d] = vs[j]; Trho[d] = p;
        }
      }
    }
    // the transition's sample starts as the starting point with its fresh momentum
    if (P.diag) copy(Sp, Wp);
    s.F_lp = s.W_lp;
    s.B_lp = s.W_lp;
    s.lsw = 0;
    s.n_leapfrog = 0;
    s.sum_metro = 0;
    s.depth = 0;
    s.divergent = 0;
    tsync<TW>();
    return begin_doubling();
  }

  __device__ bool begin_doubling() {
    s.dir = uniform() > 0.5 ? 1 : -1;
    if (s.dir > 0) load_W_from(Fq, Fp, Fg, s.F_lp);
    else load_W_from(Bq, Bp, Bg, s.B_lp);
    s.leaf = 0;
    s.free_mask = (1u << P.R) - 1u;
    s.stk_lo = ~0ull;
    s.stk_hi = ~0ull;
    begin_leapfrog(s.dir * s.eps);
    s.phase = PH_LEAF;
    return true;
  }

  // merge pending left subtree A (init) with the current subtree Bk (final);
  // result is left in A.  Returns the no-U-turn verdict.
  __device__ bool merge(int A, int Bk) {
    // record weights are finite here (a divergent leaf ends the transition
    // before any merge).  One exp serves both the log-sum-exp and the
    // probability w_B / (w_A + w_B) of taking B's proposal.
    const double lswA = rlsw(A), lswB = rlsw(Bk);
    const double x = lswB - lswA;
    double lsw_sub, a;
    if (x <= 0) {
      const double e = exp(x);
      lsw_sub = lswA + log1p(e);
      a = e / (1.0 + e);
    } else {
      const double e = exp(-x);
      lsw_sub = lswB + log1p(e);
      a = 1.0 / (1.0 + e);
    }
    const bool take = uniform() < a;
    double *Apb = rec(A, RV_PB), *Asb = rec(A, RV_SB), *Ape = rec(A, RV_PE), *Ase = rec(A, RV_SE),
           *Arho = rec(A, RV_RHO), *Aq = rec(A, RV_Q), *Ag = rec(A, RV_G);
    double *Bpb = rec(Bk, RV_PB), *Bsb = rec(Bk, RV_SB), *Bpe = rec(Bk, RV_PE), *Bse = rec(Bk, RV_SE),
           *Brho = rec(Bk, RV_RHO), *Bq_ = rec(Bk, RV_Q), *Bg_ = rec(Bk, RV_G);
    double s1a = 0, s1b = 0, s2a = 0, s2b = 0, s3a = 0, s3b = 0;
    // chunks of VCH elements per lane: all loads of a chunk are issued before
    // any of its stores (the records live in global memory and the compiler
    // cannot reorder loads across possibly aliasing stores).  Masked
    // elements load 0 and add exact zeros to the sums.
    for (int base = 0; base < D; base += TW * VCH) {
      double arho[VCH], brho[VCH], bpb[VCH], ape[VCH], asb[VCH], bse[VCH], bsb[VCH], ase[VCH], bpe[VCH];
#pragma unroll
      for (int j = 0; j < VCH; ++j) {
        const int d = base + lane + TW * j;
        const bool ok = d < D;
        arho[j] = ok ? Arho[d] : 0.0; brho[j] = ok ? Brho[d] : 0.0; bpb[j] = ok ? Bpb[d] : 0.0;
        ape[j] = ok ? Ape[d] : 0.0;   asb[j] = ok ? Asb[d] : 0.0;   bse[j] = ok ? Bse[d] : 0.0;
        bsb[j] = ok ? Bsb[d] : 0.0;   ase[j] = ok ? Ase[d] : 0.0;   bpe[j] = ok ? Bpe[d] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < VCH; ++j) {
        const double rs = arho[j] + brho[j];
        const double e1 = arho[j] + bpb[j];
        const double e2 = brho[j] + ape[j];
        s1a += asb[j] * rs;
        s1b += bse[j] * rs;
        s2a += asb[j] * e1;
        s2b += bsb[j] * e1;
        s3a += ase[j] * e2;
        s3b += bse[j] * e2;
        const int d = base + lane + TW * j;
        if (d < D) {
          Arho[d] = rs;
          Ape[d] = bpe[j];
          Ase[d] = bse[j];
        }
      }
    }
    if (take) copy2(Aq, Bq_, Ag, Bg_);
    if (take && P.diag) copy(rec(A, RV_P), rec(Bk, RV_P));
    {
      double v6[6] = {s1a, s1b, s2a, s2b, s3a, s3b};
      tsum_n<TW, 6>(v6);
      s1a = v6[0]; s1b = v6[1]; s2a = v6[2]; s2b = v6[3]; s3a = v6[4]; s3b = v6[5];
    }
    if (take) {
      const double lpB = rlp(Bk), hB = rh(Bk);
      rlp(A) = lpB;
      rh(A) = hB;
    }
    rlsw(A) = lsw_sub;
    tsync<TW>();
    return (s1b > 0 && s1a > 0) && (s2b > 0 && s2a > 0) && (s3b > 0 && s3a > 0);
  }

  // step_leaf for the diagonal and unit metrics when a chain's vectors fit one
  // chunk of VC1 elements per lane (D <= 128): the leapfrog's second half step, the leaf record and
  // -- when the doubling goes on without a merge -- the next leapfrog's first
  // half step and position update run as one pass over registers, with one
  // load of W (the separate steps take three memory round trips).  Same
  // arithmetic, element by element and in each lane's order, as
  // complete_leapfrog, the record loop of step_leaf and begin_leapfrog.
  __device__ bool step_leaf_onepass(double e) {
    ++s.n_grad;
    ++s.n_leapfrog;
    const int r = alloc_rec();
    double *pb = rec(r, RV_PB), *sb = rec(r, RV_SB), *pe = rec(r, RV_PE), *se = rec(r, RV_SE),
           *rho = rec(r, RV_RHO), *rq = rec(r, RV_Q), *rg = rec(r, RV_G);
    double* rp = P.diag ? rec(r, RV_P) : nullptr;
    double vp[VC1], vg[VC1], vq[VC1], vm[VC1];
#pragma unroll
    for (int j = 0; j < VC1; ++j) {
      const int d = lane + TW * j;
      const bool ok = d < D;
      vp[j] = ok ? Wp[d] : 0.0;
      vg[j] = ok ? Wg[d] : 0.0;
      vq[j] = ok ? Wq[d] : 0.0;
      vm[j] = ok && metric() == 0 ? minv[d] : 0.0;
    }
    double kin = 0;
#pragma unroll
    for (int j = 0; j < VC1; ++j) {
      const int d = lane + TW * j;
      if (d < D) {
        const double p = vp[j] + 0.5 * e * vg[j];
        vp[j] = p;
        Wp[d] = p;
        const double ps = metric() == 0 ? vm[j] * p : p;
        kin += p * ps;
        pb[d] = p; pe[d] = p; sb[d] = ps; se[d] = ps; rho[d] = p;
        rq[d] = vq[j]; rg[d] = vg[j];
        if (rp) rp[d] = p;
      }
    }
    double h = 0.5 * tsum<TW>(kin) - s.W_lp;
    if (isnan(h)) h = __longlong_as_double(0x7ff0000000000000ll);
    if (h - s.H0 > 1000.0) s.divergent = 1;
    s.sum_metro += (s.H0 - h > 0) ? 1.0 : exp(s.H0 - h);
    rlsw(r) = s.H0 - h;
    rlp(r) = s.W_lp;
    rh(r) = h;
    tsync<TW>();
    if (s.divergent) return end_transition();
    if (!(s.leaf & 1) && s.depth != 0) {
      // no pending subtree to merge and the doubling goes on: park the leaf at
      // height 0 and start the next leapfrog from the registers
      stack_set(0, r);
      ++s.leaf;
#pragma unroll
      for (int j = 0; j < VC1; ++j) {
        const int d = lane + TW * j;
        if (d < D) {
          const double pn = vp[j] + 0.5 * e * vg[j];
          Wp[d] = pn;
          Wq[d] = vq[j] + e * (metric() == 0 ? vm[j] * pn : pn);
        }
      }
      tsync<TW>();
      return true;
    }
    return after_leaf(r, e);
  }

  // merges of the new leaf r with the pending subtrees, then the end of the
  // doubling or the next leapfrog
  __device__ bool after_leaf(int r, double e) {
    int cur = r, height = 0;
    while ((s.leaf >> height) & 1) {
      const int A = stack_get(height);
      stack_set(height, 31);
      bool ok = merge(A, cur);
      free_rec(cur);
      cur = A;
      ++height;
      if (!ok) return end_transition();
    }
    if (height == s.depth) return finish_doubling(cur);
    stack_set(height, cur);
    ++s.leaf;
    begin_leapfrog(e);
    return true;
  }

  __device__ bool step_leaf() {
    const double e = s.dir * s.eps;
    if (metric() != 1 && D <= TW * VC1) return step_leaf_onepass(e);
    complete_leapfrog(e);
    ++s.n_leapfrog;
    int r = alloc_rec();
    double *pb = rec(r, RV_PB), *sb = rec(r, RV_SB), *pe = rec(r, RV_PE), *se = rec(r, RV_SE),
           *rho = rec(r, RV_RHO), *rq = rec(r, RV_Q), *rg = rec(r, RV_G);
    if (P.diag) copy(rec(r, RV_P), Wp);  // the leaf's proposal momentum (diagnostic rows)
    // p_sharp = minv p is formed in registers and stored to both ends of the
    // new leaf record (the dense metric needs the warp-wide product first)
    double kin = 0;
    if (metric() == 1) {
      dtau(tmp, Wp);
      for (int d = lane; d < D; d += TW) kin += Wp[d] * tmp[d];
      for (int d = lane; d < D; d += TW) {
        const double p = Wp[d];
        const double ps = tmp[d];
        pb[d] = p; pe[d] = p; sb[d] = ps; se[d] = ps; rho[d] = p;
        rq[d] = Wq[d]; rg[d] = Wg[d];
      }
    } else {
      // the leaf's kinetic energy and its record in one chunked pass
      for (int base = 0; base < D; base += TW * VCW) {
        double vp[VCW], vm[VCW], vq[VCW], vg[VCW];
#pragma unroll
        for (int j = 0; j < VCW; ++j) {
          const int d = base + lane + TW * j;
          const bool ok = d < D;
          vp[j] = ok ? Wp[d] : 0.0;
          vm[j] = ok && metric() == 0 ? minv[d] : 0.0;
          vq[j] = ok ? Wq[d] : 0.0;
          vg[j] = ok ? Wg[d] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < VCW; ++j) {
          const int d = base + lane + TW * j;
          if (d < D) {
            const double p = vp[j];
            const double ps = metric() == 0 ? vm[j] * p : p;
            kin += p * ps;
            pb[d] = p; pe[d] = p; sb[d] = ps; se[d] = ps; rho[d] = p;
            rq[d] = vq[j]; rg[d] = vg[j];
          }
        }
      }
    }
    double h = 0.5 * tsum<TW>(kin) - s.W_lp;
    if (isnan(h)) h = __longlong_as_double(0x7ff0000000000000ll);
    if (h - s.H0 > 1000.0) s.divergent = 1;
    s.sum_metro += (s.H0 - h > 0) ? 1.0 : exp(s.H0 - h);
    rlsw(r) = s.H0 - h;
    rlp(r) = s.W_lp;
    rh(r) = h;
    tsync<TW>();
    if (s.divergent) return end_transition();
    return after_leaf(r, e);
  }

  __device__ bool finish_doubling(int N) {
    if (s.dir > 0) {
      copy3(Fq, Wq, Fp, Wp, Fg, Wg); s.F_lp = s.W_lp;
    } else {
      copy3(Bq, Wq, Bp, Wp, Bg, Wg); s.B_lp = s.W_lp;
    }
    ++s.depth;
    bool take;
    // biased progressive sampling: a heavier new subtree is always taken
    const double lswN = rlsw(N);
    const double x = lswN - s.lsw;
    double lsw_new;
    if (x > 0) {
      take = true;
      lsw_new = lswN + log1p(exp(-x));
    } else {
      const double e = exp(x);
      take = uniform() < e;
      lsw_new = s.lsw + log1p(e);
    }
    double *Npb = rec(N, RV_PB), *Nsb = rec(N, RV_SB), *Npe = rec(N, RV_PE), *Nse = rec(N, RV_SE),
           *Nrho = rec(N, RV_RHO), *Nq = rec(N, RV_Q), *Ng = rec(N, RV_G);
    if (take) {
      copy2(Sq, Nq, Sg, Ng);
      if (P.diag) copy(Sp, rec(N, RV_P));
      s.S_lp = rlp(N);
      s.S_h = rh(N);
    }
    s.lsw = lsw_new;
    // In time order the trajectory is [init | final]: forward -> (T, N),
    // backward -> (N reversed, T).
    double s1a = 0, s1b = 0, s2a = 0, s2b = 0, s3a = 0, s3b = 0;
    // loads of a chunk ahead of its stores, as in merge
    for (int base = 0; base < D; base += TW * VCH) {
      double trho[VCH], tpb[VCH], tpe[VCH], tsb[VCH], tse[VCH], nrho[VCH], npb[VCH], npe[VCH], nsb[VCH], nse[VCH];
#pragma unroll
      for (int j = 0; j < VCH; ++j) {
        const int d = base + lane + TW * j;
        const bool ok = d < D;
        trho[j] = ok ? Trho[d] : 0.0; tpb[j] = ok ? Tpb[d] : 0.0; tpe[j] = ok ? Tpe[d] : 0.0;
        tsb[j] = ok ? Tsb[d] : 0.0;   tse[j] = ok ? Tse[d] : 0.0; nrho[j] = ok ? Nrho[d] : 0.0;
        npb[j] = ok ? Npb[d] : 0.0;   npe[j] = ok ? Npe[d] : 0.0; nsb[j] = ok ? Nsb[d] : 0.0;
        nse[j] = ok ? Nse[d] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < VCH; ++j) {
        const int d = base + lane + TW * j;
        if (s.dir > 0) {
          const double rs = trho[j] + nrho[j];
          const double e1 = trho[j] + npb[j];
          const double e2 = nrho[j] + tpe[j];
          s1a += tsb[j] * rs; s1b += nse[j] * rs;
          s2a += tsb[j] * e1; s2b += nsb[j] * e1;
          s3a += tse[j] * e2; s3b += nse[j] * e2;
          if (d < D) { Trho[d] = rs; Tpe[d] = npe[j]; Tse[d] = nse[j]; }
        } else {
          const double rs = nrho[j] + trho[j];
          const double e1 = nrho[j] + tpb[j];
          const double e2 = trho[j] + npb[j];
          s1a += nse[j] * rs; s1b += tse[j] * rs;
          s2a += nse[j] * e1; s2b += tsb[j] * e1;
          s3a += nsb[j] * e2; s3b += tse[j] * e2;
          if (d < D) { Trho[d] = rs; Tpb[d] = npe[j]; Tsb[d] = nse[j]; }
        }
      }
    }
    {
      double v6[6] = {s1a, s1b, s2a, s2b, s3a, s3b};
      tsum_n<TW, 6>(v6);
      s1a = v6[0]; s1b = v6[1]; s2a = v6[2]; s2b = v6[3]; s3a = v6[4]; s3b = v6[5];
    }
    free_rec(N);
    tsync<TW>();
    bool persist = (s1b > 0 && s1a > 0) && (s2b > 0 && s2a > 0) && (s3b > 0 && s3a > 0);
    if (!persist || s.depth >= P.max_depth) return end_transition();
    return begin_doubling();
  }

  __device__ void record(double accept) {
    const bool warm = s.iter < P.num_warmup;
    const int m = warm ? s.iter : s.iter - P.num_warmup;
    if ((warm && !P.save_warmup) || (m % P.thin) != 0) return;
    double* row = B.draws + ((size_t)c * P.n_saved + s.row) * P.ncol;
    if (lane == 0) {
      row[0] = s.S_lp; row[1] = accept; row[2] = s.eps; row[3] = s.depth;
      row[4] = s.n_leapfrog; row[5] = s.divergent; row[6] = s.S_h;
    }
    if (P.diag) {
      // diagnostic_file row: sampler columns, unconstrained q, momentum p, gradient
      double* dr = B.diag_draws + ((size_t)c * P.n_saved + s.row) * (7 + 3 * (size_t)P.D);
      if (lane == 0) {
        dr[0] = s.S_lp; dr[1] = accept; dr[2] = s.eps; dr[3] = s.depth;
        dr[4] = s.n_leapfrog; dr[5] = s.divergent; dr[6] = s.S_h;
      }
      for (int d = lane; d < D; d += TW) {
        dr[7 + d] = Sq[d];
        dr[7 + P.D + d] = Sp[d];
        dr[7 + 2 * P.D + d] = Sg[d];
      }
    }
    if (B.zdraws) {
      double* zr = B.zdraws + ((size_t)c * P.n_saved + s.row) * P.D;
      for (int d = lane; d < D; d += TW) zr[d] = Sq[d];
    } else {
      warp_write_array<TW>(M, Sq, row + 7, lane);
      // columns past this chain's model (a smaller member of a posterior set)
      for (int i = M.ncon + lane; i < P.ncon; i += TW) row[7 + i] = __longlong_as_double(0x7ff8000000000000ll);
    }
    ++s.row;
  }

  // returns true if a gradient is requested
  __device__ bool end_transition() {
    const double accept = s.sum_metro / (double)s.n_leapfrog;
    s.n_lf_total += s.n_leapfrog;
    tsync<TW>();
    record(accept);
    const bool warm = s.iter < P.num_warmup;
    ++s.iter;
    if (warm && P.adapt) {
      // stepsize_adaptation::learn_stepsize
      s.da_counter += 1;
      double a = accept > 1 ? 1 : accept;
      double eta = 1.0 / (s.da_counter + P.t0);
      s.da_sbar = (1.0 - eta) * s.da_sbar + eta * (P.delta - a);
      double x = s.da_mu - s.da_sbar * sqrt(s.da_counter) / P.gamma;
      double xe = pow(s.da_counter, -P.kappa);
      s.da_xbar = (1.0 - xe) * s.da_xbar + xe * x;
      s.nom_eps = exp(x);
      if (metric() != 2) {
        if (learn_metric()) {
          if (s.phase == PH_ERROR) return false;
          return begin_init_stepsize(1);
        }
      }
    }
    return begin_transition();
  }

  // windowed Welford adaptation; returns true when the metric was updated
  __device__ bool learn_metric() {
    const bool in_window = s.w_counter >= s.w_ib && s.w_counter < s.w_nw - s.w_tb && s.w_counter != s.w_nw;
    const bool end_window = s.w_counter == s.w_next && s.w_counter != s.w_nw;
    if (in_window) welford_add(end_window);  // a window end reads the estimate next
    if (!end_window) {
      ++s.w_counter;
      return false;
    }
    // compute_next_window
    if (s.w_next != s.w_nw - s.w_tb - 1) {
      s.w_size *= 2;
      s.w_next = s.w_counter + s.w_size;
      if (s.w_next != s.w_nw - s.w_tb - 1) {
        unsigned boundary = s.w_next + 2 * s.w_size;
        if (boundary >= s.w_nw - s.w_tb) s.w_next = s.w_nw - s.w_tb - 1;
      }
    }
    const double n = s.wf_n;
    bool ok = true;
    if (metric() == 1) {
      for (int i = 0; i < D; ++i)
        for (int j = lane; j < D; j += TW) {
          const size_t ij = (size_t)i * P.ld + j;
          double v = (dense32() ? (double)w32[ij] + (double)w32lo[ij] : wm2[ij]) / (n - 1.0);
          v = (n / (n + 5.0)) * v + (i == j ? 1e-3 * (5.0 / (n + 5.0)) : 0.0);
          minv[ij] = v;
          if (dense32()) m32[ij] = (float)v;
          ok = ok && isfinite(v);
        }
    } else {
      for (int d = lane; d < D; d += TW) {
        double v = wm2[d] / (n - 1.0);
        v = (n / (n + 5.0)) * v + 1e-3 * (5.0 / (n + 5.0));
        minv[d] = v;
        ok = ok && isfinite(v);
      }
    }
    tsync<TW>();
    if (!tall<TW>(ok)) { fail(CE_METRIC); return true; }
    if (metric() == 1 && !cholesky()) { fail(CE_NOT_PD); return true; }
    if (dense32()) copy_chol32();
    // restart the estimator
    s.wf_n = 0;
    for (int d = lane; d < D; d += TW) wm[d] = 0;
    if (dense32()) {
      for (int i = 0; i < D; ++i)
        for (int j = lane; j < D; j += TW) {
          w32[(size_t)i * P.ld + j] = 0.f;
          w32lo[(size_t)i * P.ld + j] = 0.f;
        }
    } else if (metric() == 1) {
      for (int i = 0; i < D; ++i)
        for (int j = lane; j < D; j += TW) wm2[(size_t)i * P.ld + j] = 0;
    } else {
      for (int d = lane; d < D; d += TW) wm2[d] = 0;
    }
    ++s.w_counter;
    tsync<TW>();
    return true;
  }

  __device__ void welford_add(bool local) {
    s.wf_n += 1;
    const double n = s.wf_n;
    for (int d = lane; d < D; d += TW) {
      double q = Sq[d];
      double delta = q - wm[d];
      wm[d] += delta / n;
      if (metric() == 1) tmp[d] = delta;
      else wm2[d] += (q - wm[d]) * delta;
    }
    if (dense32()) {
      // wm2 += a b^T with a = q - mean (updated), b = q - mean (previous), in
      // float-float arithmetic (about 44 significant bits): an FP32 sum's
      // rounding, relative to the large variances of a wide posterior, can
      // exceed the 1e-3 (5 / (n + 5)) ridge of a short window and leave the
      // estimate indefinite.  a and b are split into float pairs; the D x D
      // update is applied here at a window end (the estimate is read next),
      // otherwise queued for k_welford_dense, which runs the round's queued
      // updates over every SM instead of this chain's one.
      float* bh = local ? fbuf() : B.wpend + (size_t)c * 4 * P.ld;
      const int st = local ? DENSE32_MAXD : P.ld;
      float* bl = bh + st;
      float* ah = bh + 2 * st;
      float* al = bh + 3 * st;
      tsync<TW>();
      for (int d = lane; d < D; d += TW) {
        const double b = tmp[d], a = Sq[d] - wm[d];
        const float hb = (float)b, ha = (float)a;
        bh[d] = hb;
        bl[d] = (float)(b - (double)hb);
        ah[d] = ha;
        al[d] = (float)(a - (double)ha);
      }
      tsync<TW>();
      if (local) {
        for (int i = 0; i < D; ++i) {
          const float a0 = ah[i], a1 = al[i];
          float* wr = w32 + (size_t)i * P.ld;
          float* wl = w32lo + (size_t)i * P.ld;
          for (int j = lane; j < D; j += TW) ff_axpy(wr[j], wl[j], a0, a1, bh[j], bl[j]);
        }
      } else if (lane == 0) {
        const int k = atomicAdd(B.wlist, 1);
        B.wlist[2 + k] = c;
      }
    } else if (metric() == 1) {
      tsync<TW>();
      for (int i = 0; i < D; ++i) {
        double a = Sq[i] - wm[i];
        for (int j = lane; j < D; j += TW) wm2[(size_t)i * P.ld + j] += a * tmp[j];
      }
    }
    tsync<TW>();
  }

  // Lt (row k holds column k of L) from minv; false if not positive definite
  __device__ bool cholesky() {
    for (int j = 0; j < D; ++j) {
      double* Lj = chol + (size_t)j * P.ld;  // Lt row j = L column j
      double t = 0;
      if constexpr (TW > 32) {
        // a team sums the column's squares in parallel (one warp keeps the
        // serial order, as the reference's factorisation does)
        for (int k = lane; k < j; k += TW) {
          const double l = chol[(size_t)k * P.ld + j];
          t += l * l;
        }
        t = tsum<TW>(t);
      } else {
        for (int k = 0; k < j; ++k) {
          double l = chol[(size_t)k * P.ld + j];
          t += l * l;
        }
      }
      double sdiag = minv[(size_t)j * P.ld + j] - t;
      if (!(sdiag > 0)) return false;
      double dj = sqrt(sdiag);
      for (int i = j + 1 + lane; i < D; i += TW) {
        double u = minv[(size_t)i * P.ld + j];
        for (int k = 0; k < j; ++k) u -= chol[(size_t)k * P.ld + i] * chol[(size_t)k * P.ld + j];
        Lj[i] = u / dj;
      }
      if (lane == 0) Lj[j] = dj;
      for (int i = lane; i < j; i += TW) Lj[i] = 0.0;
      tsync<TW>();
    }
    return true;
  }
  __device__ void copy_chol32() {
    for (int i = 0; i < D; ++i)
      for (int j = lane; j < D; j += TW) l32[(size_t)i * P.ld + j] = (float)chol[(size_t)i * P.ld + j];
    tsync<TW>();
  }

  // ---------------- driver ----------------
  __device__ __forceinline__ bool advance() {
    switch (s.phase) {
      case PH_INIT: {
        if (W_finite()) {
          copy(Sq, Wq);
          copy(Sg, Wg);
          s.S_lp = s.W_lp;
          ++s.n_grad;
          tsync<TW>();
          if (P.adapt) return begin_init_stepsize(0);
          return begin_transition();
        }
        ++s.n_grad;
        const int max_attempts = (P.has_init || P.init_radius == 0) ? 1 : 100;
        if (s.init_attempts >= max_attempts) { fail(CE_INIT); return false; }
        init_candidate();
        return true;
      }
      case PH_IS_FIRST:
      case PH_IS_LOOP:
        return step_init_stepsize();
      case PH_LEAF:
        return step_leaf();
      default:
        return false;
    }
  }
};

// replay inputs of the transition-level entry point (chain ids, RNG offsets)
struct ReplayBufs {
  const unsigned* chain_ids;
  const unsigned long long* rng_start;
};

// fused.cu / fused_kind.cu: the fused-mode kernel, one instantiation per
// model kind (only that model's gradient is compiled into it)
template <int KIND>
cudaError_t fused_set_smem_k(int bytes);
template <int KIND>
cudaError_t fused_launch_k(int blocks, int threads, size_t smem, const Params& P, const Bufs& B, const DevModel& M,
                           const ReplayBufs& RB);
cudaError_t fused_set_smem(int kind, int bytes);
cudaError_t fused_launch(int kind, int blocks, int threads, size_t smem, const Params& P, const Bufs& B,
                         const DevModel& M, const ReplayBufs& RB);

}  // namespace gnuts

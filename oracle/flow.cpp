// CPU FP64 restatement of the affine-coupling flow -- TEST INFRASTRUCTURE ONLY.
//
// The learned preconditioner has no counterpart in the reference (CmdStan
// samples the model's own unconstrained space); this file restates, in plain
// FP64 loops, the map the device kernels implement, so their forward,
// inverse, log-determinant, input gradient, parameter gradient and Adam step
// can be checked.  Published method: RealNVP affine coupling layers (Dinh,
// Sohl-Dickstein & Bengio 2017) with a tanh hidden layer and a soft-clamped
// log-scale; Adam (Kingma & Ba 2015).
//
// Map (z -> x), d dimensions, L layers, H hidden units:
//   u_0 = z;  u_{l+1} = f_l(u_l);  x = mu + exp(rho) .* u_L
//   f_l: the dimensions split into a conditioner set b_l and a transformed
//        set a_l (bit k = l mod B of the index equals polarity (l / B) mod 2
//        for members of b_l, B = ceil(log2 d));
//        pre = W1^T u_b + b1 (H), h = tanh(pre), r = W2^T h + b2 (2 n_a),
//        s = c tanh(r_s / c), y_a = u_a .* exp(s) + r_t, y_b = u_b.
//   log|det dx/dz| = sum_l sum s_l + sum rho.
// Parameter vector theta, per layer: W1 [n_b][H], b1 [H], W2 [H][2 n_a],
// b2 [2 n_a]; then mu [d], rho [d].  Row r of W1 belongs to the r-th member
// of b_l in increasing order; column m < n_a of W2 is the log-scale of the
// m-th member of a_l, column n_a + m its shift.
#include <cmath>
#include <cstring>
#include <vector>
#include "oracle.h"

namespace {

struct Shape {
  int d, L, H;
  std::vector<std::vector<int>> b, a;
  std::vector<long> off;  // per layer: offset of W1 (b1, W2, b2 follow)
  long off_mu, off_rho, n;
};

Shape make_shape(int d, int L, int H) {
  Shape S;
  S.d = d;
  S.L = L;
  S.H = H;
  int B = 0;
  while ((1 << B) < d) ++B;
  if (B == 0) B = 1;
  long o = 0;
  for (int l = 0; l < L; ++l) {
    const int k = l % B, pol = (l / B) & 1;
    std::vector<int> bl, al;
    for (int i = 0; i < d; ++i) (((i >> k) & 1) == pol ? bl : al).push_back(i);
    S.b.push_back(bl);
    S.a.push_back(al);
    S.off.push_back(o);
    o += (long)bl.size() * H + H + (long)H * 2 * al.size() + 2 * (long)al.size();
  }
  S.off_mu = o;
  S.off_rho = o + d;
  S.n = o + 2 * d;
  return S;
}

struct Tape {
  // per layer: input u (d), hidden h (H), log-scale s (n_a), output y (d)
  std::vector<std::vector<double>> u, h, s;
  std::vector<double> uL;
};

// forward map with the tape; returns log|det|
double forward(const Shape& S, double clamp, const double* th, const double* z, double* x, Tape* T) {
  std::vector<double> u(z, z + S.d);
  double logdet = 0;
  if (T) {
    T->u.assign(S.L, {});
    T->h.assign(S.L, {});
    T->s.assign(S.L, {});
  }
  for (int l = 0; l < S.L; ++l) {
    const auto &b = S.b[l], &a = S.a[l];
    const int nb = (int)b.size(), na = (int)a.size(), H = S.H;
    const double* W1 = th + S.off[l];
    const double* b1 = W1 + (long)nb * H;
    const double* W2 = b1 + H;
    const double* b2 = W2 + (long)H * 2 * na;
    std::vector<double> h(H), s(na), t(na);
    for (int j = 0; j < H; ++j) {
      double p = b1[j];
      for (int r = 0; r < nb; ++r) p += W1[(long)r * H + j] * u[b[r]];
      h[j] = std::tanh(p);
    }
    for (int m = 0; m < na; ++m) {
      double rs = b2[m], rt = b2[na + m];
      for (int j = 0; j < H; ++j) {
        rs += W2[(long)j * 2 * na + m] * h[j];
        rt += W2[(long)j * 2 * na + na + m] * h[j];
      }
      s[m] = clamp * std::tanh(rs / clamp);
      t[m] = rt;
    }
    if (T) {
      T->u[l] = u;
      T->h[l] = h;
      T->s[l] = s;
    }
    for (int m = 0; m < na; ++m) {
      u[a[m]] = u[a[m]] * std::exp(s[m]) + t[m];
      logdet += s[m];
    }
  }
  if (T) T->uL = u;
  const double* mu = th + S.off_mu;
  const double* rho = th + S.off_rho;
  for (int i = 0; i < S.d; ++i) {
    x[i] = mu[i] + std::exp(rho[i]) * u[i];
    logdet += rho[i];
  }
  return logdet;
}

// adjoint sweep: given xbar = d(objective)/dx, adds the log-determinant's
// own derivative (objective = f(x) + log|det|) and returns zbar; accumulates
// d(objective)/dtheta into thbar when non-null
void backward(const Shape& S, double clamp, const double* th, const Tape& T, const double* xbar, double* zbar,
              double* thbar) {
  const double* rho = th + S.off_rho;
  std::vector<double> y(S.d);
  for (int i = 0; i < S.d; ++i) {
    y[i] = xbar[i] * std::exp(rho[i]);
    if (thbar) {
      thbar[S.off_mu + i] += xbar[i];
      thbar[S.off_rho + i] += xbar[i] * std::exp(rho[i]) * T.uL[i] + 1.0;
    }
  }
  for (int l = S.L - 1; l >= 0; --l) {
    const auto &b = S.b[l], &a = S.a[l];
    const int nb = (int)b.size(), na = (int)a.size(), H = S.H;
    const double* W1 = th + S.off[l];
    const double* b1 = W1 + (long)nb * H;
    const double* W2 = b1 + H;
    const std::vector<double>& u = T.u[l];
    const std::vector<double>& h = T.h[l];
    const std::vector<double>& s = T.s[l];
    std::vector<double> rbar(2 * na), ubar(S.d, 0.0);
    for (int m = 0; m < na; ++m) {
      const double ys = y[a[m]];
      const double es = std::exp(s[m]);
      ubar[a[m]] = ys * es;
      const double sbar = ys * u[a[m]] * es + 1.0;
      const double q = s[m] / clamp;
      rbar[m] = sbar * (1.0 - q * q);
      rbar[na + m] = ys;
    }
    std::vector<double> pbar(H);
    for (int j = 0; j < H; ++j) {
      double hb = 0;
      for (int m = 0; m < 2 * na; ++m) hb += W2[(long)j * 2 * na + m] * rbar[m];
      pbar[j] = hb * (1.0 - h[j] * h[j]);
    }
    for (int r = 0; r < nb; ++r) {
      double t = y[b[r]];
      for (int j = 0; j < H; ++j) t += W1[(long)r * H + j] * pbar[j];
      ubar[b[r]] = t;
    }
    if (thbar) {
      double* gW1 = thbar + S.off[l];
      double* gb1 = gW1 + (long)nb * H;
      double* gW2 = gb1 + H;
      double* gb2 = gW2 + (long)H * 2 * na;
      for (int r = 0; r < nb; ++r)
        for (int j = 0; j < H; ++j) gW1[(long)r * H + j] += u[b[r]] * pbar[j];
      for (int j = 0; j < H; ++j) gb1[j] += pbar[j];
      for (int j = 0; j < H; ++j)
        for (int m = 0; m < 2 * na; ++m) gW2[(long)j * 2 * na + m] += h[j] * rbar[m];
      for (int m = 0; m < 2 * na; ++m) gb2[m] += rbar[m];
    }
    y = ubar;
  }
  std::memcpy(zbar, y.data(), sizeof(double) * S.d);
}

}  // namespace

extern "C" {

long orc_flow_num_params(int d, int L, int H) { return make_shape(d, L, H).n; }

/* conditioner set membership of layer l: out[i] = 1 if i is in b_l */
void orc_flow_mask(int d, int L, int H, int l, int* out) {
  Shape S = make_shape(d, L, H);
  for (int i = 0; i < d; ++i) out[i] = 0;
  for (int i : S.b[l]) out[i] = 1;
}

double orc_flow_forward(int d, int L, int H, double clamp, const double* theta, const double* z, double* x) {
  Shape S = make_shape(d, L, H);
  return forward(S, clamp, theta, z, x, nullptr);
}

double orc_flow_inverse(int d, int L, int H, double clamp, const double* theta, const double* x, double* z) {
  Shape S = make_shape(d, L, H);
  const double* mu = theta + S.off_mu;
  const double* rho = theta + S.off_rho;
  std::vector<double> y(d);
  double logdet = 0;
  for (int i = 0; i < d; ++i) {
    y[i] = (x[i] - mu[i]) * std::exp(-rho[i]);
    logdet += rho[i];
  }
  for (int l = L - 1; l >= 0; --l) {
    const auto &b = S.b[l], &a = S.a[l];
    const int nb = (int)b.size(), na = (int)a.size();
    const double* W1 = theta + S.off[l];
    const double* b1 = W1 + (long)nb * H;
    const double* W2 = b1 + H;
    const double* b2 = W2 + (long)H * 2 * na;
    std::vector<double> h(H);
    for (int j = 0; j < H; ++j) {
      double p = b1[j];
      for (int r = 0; r < nb; ++r) p += W1[(long)r * H + j] * y[b[r]];
      h[j] = std::tanh(p);
    }
    for (int m = 0; m < na; ++m) {
      double rs = b2[m], rt = b2[na + m];
      for (int j = 0; j < H; ++j) {
        rs += W2[(long)j * 2 * na + m] * h[j];
        rt += W2[(long)j * 2 * na + na + m] * h[j];
      }
      const double s = clamp * std::tanh(rs / clamp);
      y[a[m]] = (y[a[m]] - rt) * std::exp(-s);
      logdet += s;
    }
  }
  std::memcpy(z, y.data(), sizeof(double) * d);
  return logdet;
}

/* log density of the pulled-back target at z: lp_x(T(z)) + log|det| (jacobian
 * of the model's own constraining transforms as `jacobian`), its gradient in
 * z, and (thbar non-null) its gradient in theta, accumulated.  x_out (may be
 * null) receives T(z); lp_x_out (may be null) the model's lp at T(z). */
double orc_flow_log_prob_grad(const orc_model* m, int L, int H, double clamp, const double* theta,
                              const double* z, int jacobian, double* grad_z, double* thbar, double* x_out,
                              double* lp_x_out) {
  const int d = orc_model_dim(m);
  Shape S = make_shape(d, L, H);
  Tape T;
  std::vector<double> x(d), gx(d);
  const double logdet = forward(S, clamp, theta, z, x.data(), &T);
  const double lpx = orc_log_prob_grad(m, x.data(), jacobian, gx.data());
  backward(S, clamp, theta, T, gx.data(), grad_z, thbar);
  if (x_out) std::memcpy(x_out, x.data(), sizeof(double) * d);
  if (lp_x_out) *lp_x_out = lpx;
  return lpx + logdet;
}

/* one Adam step (Kingma & Ba 2015, bias-corrected) on n parameters at step t >= 1 */
void orc_adam(long n, double* theta, double* m, double* v, const double* g, int t, double lr, double b1,
              double b2, double eps) {
  const double c1 = 1.0 - std::pow(b1, t), c2 = 1.0 - std::pow(b2, t);
  for (long i = 0; i < n; ++i) {
    m[i] = b1 * m[i] + (1.0 - b1) * g[i];
    v[i] = b2 * v[i] + (1.0 - b2) * g[i] * g[i];
    theta[i] -= lr * (m[i] / c1) / (std::sqrt(v[i] / c2) + eps);
  }
}

}  // extern "C"

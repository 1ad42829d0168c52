"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product never does.  See oracle.h for what the oracle
restates and how it is pinned.
"""
import ctypes
import os
import subprocess
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class Args(ctypes.Structure):
    _fields_ = [("num_warmup", ctypes.c_int), ("num_samples", ctypes.c_int), ("thin", ctypes.c_int),
                ("save_warmup", ctypes.c_int), ("stepsize", ctypes.c_double),
                ("stepsize_jitter", ctypes.c_double), ("max_depth", ctypes.c_int),
                ("adapt_engaged", ctypes.c_int), ("delta", ctypes.c_double), ("gamma", ctypes.c_double),
                ("kappa", ctypes.c_double), ("t0", ctypes.c_double), ("init_buffer", ctypes.c_uint),
                ("term_buffer", ctypes.c_uint), ("window", ctypes.c_uint), ("metric", ctypes.c_int),
                ("seed", ctypes.c_uint32), ("init_radius", ctypes.c_double)]


def args(**kw):
    a = Args(num_warmup=1000, num_samples=1000, thin=1, save_warmup=0, stepsize=1.0, stepsize_jitter=0.0,
             max_depth=10, adapt_engaged=1, delta=0.8, gamma=0.05, kappa=0.75, t0=10.0, init_buffer=75,
             term_buffer=50, window=25, metric=0, seed=0, init_radius=2.0)
    for k, v in kw.items():
        setattr(a, k, v)
    return a


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            subprocess.run(["make", "-s", "-C", HERE], check=True)
        L = ctypes.CDLL(LIB)
        vp = ctypes.c_void_p
        for f in ("orc_bernoulli", "orc_normal", "orc_logistic", "orc_hier", "orc_funnel", "orc_varint",
                  "orc_horseshoe"):
            getattr(L, f).restype = vp
        L.orc_bernoulli.argtypes = [ctypes.c_int, _ip]
        L.orc_normal.argtypes = [ctypes.c_int, _dp]
        L.orc_logistic.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _ip]
        L.orc_hier.argtypes = [ctypes.c_int, _dp, _dp]
        L.orc_funnel.argtypes = [ctypes.c_int]
        L.orc_varint.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _ip, _dp, _dp]
        L.orc_horseshoe.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _ip, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double]
        L.orc_model_free.argtypes = [vp]
        L.orc_model_dim.argtypes = [vp]
        L.orc_model_num_constrained.argtypes = [vp]
        L.orc_log_prob_grad.argtypes = [vp, _dp, ctypes.c_int, _dp]
        L.orc_log_prob_grad.restype = ctypes.c_double
        L.orc_write_array.argtypes = [vp, _dp, _dp]
        L.orc_unconstrain.argtypes = [vp, _dp, _dp]
        L.orc_run_chain.argtypes = [vp, ctypes.POINTER(Args), ctypes.c_uint32, _dp, _dp, _dp, _dp, _dp,
                                    ctypes.POINTER(ctypes.c_longlong), ctypes.c_char_p, ctypes.c_int]
        L.orc_run_chains.argtypes = [vp, ctypes.POINTER(Args), ctypes.c_int, ctypes.c_uint32, ctypes.c_int, _dp,
                                     _dp, _dp, _dp, _dp, ctypes.POINTER(ctypes.c_longlong)]
        L.orc_transition.argtypes = [vp, ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, ctypes.c_int,
                                     ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64), _dp, _dp]
        for f in ("orc_ess_bulk", "orc_ess_tail", "orc_ess_basic", "orc_rhat"):
            getattr(L, f).argtypes = [_dp, ctypes.c_int, ctypes.c_int]
            getattr(L, f).restype = ctypes.c_double
        L.orc_summary.argtypes = [_dp, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, _dp]
        L.orc_philox4x32_10.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                                        ctypes.POINTER(ctypes.c_uint32)]
        L.orc_uniform.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64]
        L.orc_uniform.restype = ctypes.c_double
        L.orc_normal_pair.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, _dp]
        L.orc_flow_num_params.argtypes = [ctypes.c_int] * 3
        L.orc_flow_num_params.restype = ctypes.c_long
        L.orc_flow_mask.argtypes = [ctypes.c_int] * 4 + [_ip]
        for f in ("orc_flow_forward", "orc_flow_inverse"):
            getattr(L, f).argtypes = [ctypes.c_int] * 3 + [ctypes.c_double, _dp, _dp, _dp]
            getattr(L, f).restype = ctypes.c_double
        L.orc_flow_log_prob_grad.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp, _dp,
                                             ctypes.c_int, _dp, _dp, _dp, _dp]
        L.orc_flow_log_prob_grad.restype = ctypes.c_double
        L.orc_adam.argtypes = [ctypes.c_long, _dp, _dp, _dp, _dp, ctypes.c_int] + [ctypes.c_double] * 4
        _lib = L
    return _lib


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class OracleModel:
    """Oracle twin of a built-in model, constructed from the same data dict."""

    def __init__(self, model_id, data):
        L = load()
        self._keep = []
        d = data
        if model_id == "bernoulli":
            y = _i(d["y"]); self._keep.append(y)
            h = L.orc_bernoulli(len(y), y.ctypes.data_as(_ip))
        elif model_id in ("normal", "proper", "test_model"):
            s = _d({"proper": [1.0], "test_model": [10.0, 1.0]}.get(model_id, d.get("scales", [1.0])))
            self._keep.append(s)
            h = L.orc_normal(len(s), s.ctypes.data_as(_dp))
        elif model_id == "logistic":
            X = _d(d["X"]); y = _i(d["y"]); self._keep += [X, y]
            h = L.orc_logistic(X.shape[0], X.shape[1], X.ctypes.data_as(_dp), y.ctypes.data_as(_ip))
        elif model_id == "hier":
            y = _d(d["y"]); s = _d(d["sigma"]); self._keep += [y, s]
            h = L.orc_hier(len(y), y.ctypes.data_as(_dp), s.ctypes.data_as(_dp))
        elif model_id == "funnel":
            h = L.orc_funnel(int(d.get("K", 100)))
        elif model_id == "varint":
            g = _i(d["group"]); X = _d(d["X"]); y = _d(d["y"])
            order = np.argsort(g, kind="stable")
            g, X, y = _i(g[order]), _d(X[order]), _d(y[order])
            self._keep += [g, X, y]
            h = L.orc_varint(len(y), int(d["J"]), int(d["K"]), g.ctypes.data_as(_ip), X.ctypes.data_as(_dp),
                             y.ctypes.data_as(_dp))
        elif model_id == "horseshoe":
            X = _d(d["X"]); y = _i(d["y"]); self._keep += [X, y]
            h = L.orc_horseshoe(X.shape[0], X.shape[1], X.ctypes.data_as(_dp), y.ctypes.data_as(_ip),
                                float(d.get("scale_global", 0.01)), float(d.get("slab_scale", 2.0)),
                                float(d.get("slab_df", 4.0)))
        else:
            raise ValueError(model_id)
        self._h = ctypes.c_void_p(h)
        self._L = L
        self.dim = L.orc_model_dim(self._h)
        self.num_constrained = L.orc_model_num_constrained(self._h)

    def __del__(self):
        if getattr(self, "_h", None) is not None:
            self._L.orc_model_free(self._h)
            self._h = None

    def log_prob_grad(self, q, jacobian=True):
        q = _d(q)
        g = np.zeros(self.dim)
        lp = self._L.orc_log_prob_grad(self._h, q.ctypes.data_as(_dp), int(jacobian), g.ctypes.data_as(_dp))
        return lp, g

    def write_array(self, q):
        q = _d(q)
        out = np.zeros(self.num_constrained)
        self._L.orc_write_array(self._h, q.ctypes.data_as(_dp), out.ctypes.data_as(_dp))
        return out

    def run_chains(self, n_chains, threads=1, first_chain_id=1, inits=None, inv_metric=None, **kw):
        a = args(**kw)
        D = self.dim
        n_saved = ((a.num_warmup + a.thin - 1) // a.thin if a.save_warmup else 0) + \
                  (a.num_samples + a.thin - 1) // a.thin
        draws = np.zeros((n_chains, n_saved, 7 + D))
        eps = np.zeros(n_chains)
        msz = D * D if a.metric == 1 else D
        minv = np.zeros((n_chains, msz))
        ng = np.zeros(n_chains, dtype=np.int64)
        ini = None if inits is None else _d(np.broadcast_to(inits, (n_chains, D)))
        im = None if inv_metric is None else _d(np.broadcast_to(np.ravel(inv_metric), (n_chains, msz)))
        rc = self._L.orc_run_chains(self._h, ctypes.byref(a), n_chains, first_chain_id, threads,
                                    None if ini is None else ini.ctypes.data_as(_dp),
                                    None if im is None else im.ctypes.data_as(_dp),
                                    draws.ctypes.data_as(_dp), eps.ctypes.data_as(_dp), minv.ctypes.data_as(_dp),
                                    ng.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)))
        if rc:
            raise RuntimeError("oracle sampler failed with code %d" % rc)
        return draws, eps, minv, ng

    def transition(self, q0, p0, eps, inv_metric=None, metric=0, max_depth=10, seed=0, chain=1, counter=0):
        q0, p0 = _d(q0), _d(p0)
        im = None if inv_metric is None else _d(inv_metric)
        c = ctypes.c_uint64(counter)
        qo = np.zeros(self.dim)
        st = np.zeros(7)
        self._L.orc_transition(self._h, metric, None if im is None else im.ctypes.data_as(_dp),
                               q0.ctypes.data_as(_dp), p0.ctypes.data_as(_dp), eps, max_depth, seed, chain,
                               ctypes.byref(c), qo.ctypes.data_as(_dp), st.ctypes.data_as(_dp))
        return qo, st, c.value


def summary(x, probs=(0.05, 0.5, 0.95)):
    """x: [chains, draws] -> dict of mean, mcse, sd, mad, quantiles, ess_bulk, ess_tail, rhat."""
    L = load()
    x = _d(np.atleast_2d(x))
    p = _d(probs)
    out = np.zeros(7 + len(p))
    L.orc_summary(x.ctypes.data_as(_dp), x.shape[0], x.shape[1], p.ctypes.data_as(_dp), len(p),
                  out.ctypes.data_as(_dp))
    r = {"mean": out[0], "mcse": out[1], "sd": out[2], "mad": out[3]}
    for i, pr in enumerate(probs):
        r["q%g" % (100 * pr)] = out[4 + i]
    r["ess_bulk"], r["ess_tail"], r["rhat"] = out[4 + len(p)], out[5 + len(p)], out[6 + len(p)]
    return r


def ess_bulk(x):
    x = _d(np.atleast_2d(x))
    return load().orc_ess_bulk(x.ctypes.data_as(_dp), x.shape[0], x.shape[1])


def rhat(x):
    x = _d(np.atleast_2d(x))
    return load().orc_rhat(x.ctypes.data_as(_dp), x.shape[0], x.shape[1])


def philox(ctr, key):
    L = load()
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    L.orc_philox4x32_10(c, k, o)
    return list(o)


class OracleFlow:
    """FP64 twin of the affine-coupling flow (flow.cpp): theta is a flat
    parameter vector in the layout documented there."""

    def __init__(self, d, layers=8, hidden=128, clamp=4.0):
        self.d, self.L, self.H, self.clamp = d, layers, hidden, float(clamp)
        self.n_params = load().orc_flow_num_params(d, layers, hidden)

    def mask(self, layer):
        out = np.zeros(self.d, dtype=np.int32)
        load().orc_flow_mask(self.d, self.L, self.H, layer, out.ctypes.data_as(_ip))
        return out

    def forward(self, theta, z):
        th, z = _d(theta), _d(z)
        x = np.zeros(self.d)
        ld = load().orc_flow_forward(self.d, self.L, self.H, self.clamp, th.ctypes.data_as(_dp),
                                     z.ctypes.data_as(_dp), x.ctypes.data_as(_dp))
        return x, ld

    def inverse(self, theta, x):
        th, x = _d(theta), _d(x)
        z = np.zeros(self.d)
        ld = load().orc_flow_inverse(self.d, self.L, self.H, self.clamp, th.ctypes.data_as(_dp),
                                     x.ctypes.data_as(_dp), z.ctypes.data_as(_dp))
        return z, ld

    def log_prob_grad(self, model, theta, z, jacobian=True, param_grad=False):
        """lp_z = lp_x(T(z)) + log|det|, d lp_z / dz and (param_grad) d lp_z / dtheta."""
        th, z = _d(theta), _d(z)
        gz = np.zeros(self.d)
        gth = np.zeros(self.n_params) if param_grad else None
        x = np.zeros(self.d)
        lpx = ctypes.c_double()
        lp = load().orc_flow_log_prob_grad(model._h, self.L, self.H, self.clamp, th.ctypes.data_as(_dp),
                                           z.ctypes.data_as(_dp), int(jacobian), gz.ctypes.data_as(_dp),
                                           None if gth is None else gth.ctypes.data_as(_dp),
                                           x.ctypes.data_as(_dp), ctypes.byref(lpx))
        return (lp, gz, gth, x, lpx.value) if param_grad else (lp, gz)


def adam(theta, m, v, g, t, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """In-place Adam step on FP64 arrays (oracle of the device Adam kernel)."""
    for a in (theta, m, v):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    g = _d(g)
    load().orc_adam(len(theta), theta.ctypes.data_as(_dp), m.ctypes.data_as(_dp), v.ctypes.data_as(_dp),
                    g.ctypes.data_as(_dp), int(t), lr, b1, b2, eps)

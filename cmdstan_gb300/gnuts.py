"""Python mirror of the gnuts C ABI (include/gnuts.h), through ctypes.

This mirrors the reference's sampling-service interface for Python callers
and tests: ``Model`` stands for a stanc-generated ``model_base`` built from a
var_context (src/cmdstan/command.hpp:165-171), and ``Model.sample`` calls the
``hmc_nuts_{diag,dense,unit}_e[_adapt]`` service that command() dispatches to
(command.hpp:609-697), with CmdStan's argument names and defaults.

The shared library is required: importing works without it, but every call
that needs it raises ``GnutsError`` (there is no CPU fallback).
"""
import ctypes
import os
import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgnuts.so")

GNUTS_OK = 0
ERR_ARGUMENT, ERR_DATA, ERR_INIT, ERR_SAMPLER, ERR_CUDA, ERR_TIMEOUT = 1, 2, 3, 4, 5, 6
PRECISION_FP64, PRECISION_MIXED = 0, 1
VAR_INT, VAR_REAL = 0, 1
SAMPLER_COLUMNS = ["lp__", "accept_stat__", "stepsize__", "treedepth__", "n_leapfrog__", "divergent__",
                   "energy__"]
METRICS = {"diag_e": 0, "dense_e": 1, "unit_e": 2}

# every symbol declared in include/gnuts.h
EXPORTS = [
    "gnuts_model_create", "gnuts_model_create_json", "gnuts_model_destroy", "gnuts_model_dims",
    "gnuts_model_name", "gnuts_model_param_name", "gnuts_log_prob_grad", "gnuts_unconstrain",
    "gnuts_write_array", "gnuts_sample_args_default", "gnuts_log_prob_grad_precision", "gnuts_hmc_nuts_diag_e_adapt",
    "gnuts_hmc_nuts_dense_e_adapt", "gnuts_hmc_nuts_unit_e_adapt", "gnuts_hmc_nuts_diag_e",
    "gnuts_hmc_nuts_dense_e", "gnuts_hmc_nuts_unit_e", "gnuts_transition", "gnuts_last_error",
    "gnuts_version", "gnuts_summary", "gnuts_summary_columns", "gnuts_log_prob_grad_noalloc",
    "gnuts_flow_create", "gnuts_flow_destroy", "gnuts_flow_num_params", "gnuts_flow_set_params",
    "gnuts_flow_get_params", "gnuts_flow_init_affine", "gnuts_flow_forward", "gnuts_flow_inverse",
    "gnuts_flow_log_prob_grad", "gnuts_flow_log_prob_grad_tc", "gnuts_flow_adam_step", "gnuts_flow_train", "gnuts_hmc_nuts_flow_diag_e_adapt",
    "gnuts_learned_args_default", "gnuts_hmc_nuts_learned_diag_e_adapt", "gnuts_train_args_default",
    "gnuts_summary_columns_gpu",
    "gnuts_diagnose", "gnuts_set_interrupt", "gnuts_set_draw_sink",
]
SUMMARY_FIELDS = ["mean", "mcse", "sd", "mad"]


def summary(x, probs=(0.05, 0.5, 0.95)):
    """stansummary statistics of one quantity; x is [chains, draws]."""
    lib = load()
    x = np.ascontiguousarray(np.atleast_2d(x), dtype=np.float64)
    p = np.ascontiguousarray(probs, dtype=np.float64)
    out = np.zeros(7 + len(p))
    _check(lib.gnuts_summary(_dp(x), x.shape[0], x.shape[1], x.shape[1], 1, _dp(p), len(p), _dp(out)))
    return _summary_dict(out, probs)


def _summary_dict(out, probs):
    r = dict(zip(SUMMARY_FIELDS, out[:4]))
    for i, pr in enumerate(probs):
        r["q%g" % (100 * pr)] = out[4 + i]
    n = len(probs)
    r["ess_bulk"], r["ess_tail"], r["rhat"] = out[4 + n], out[5 + n], out[6 + n]
    return r


def summary_columns(draws, cols, probs=(0.05, 0.5, 0.95), threads=0, gpu=False):
    """stansummary statistics of several columns of a [chains, draws, columns]
    array; gpu=True computes them on the device (gnuts_summary_columns_gpu)."""
    lib = load()
    d = np.ascontiguousarray(draws, dtype=np.float64)
    C, n, K = d.shape
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    p = np.ascontiguousarray(probs, dtype=np.float64)
    out = np.zeros((len(cols), 7 + len(p)))
    ci = cols.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    if gpu:
        rc = lib.gnuts_summary_columns_gpu(_dp(d), C, n, len(cols), n * K, K, ci, _dp(p), len(p), _dp(out))
        if rc != GNUTS_OK:
            raise GnutsError(rc, "device summary failed (code %d)" % rc)
    else:
        _check(lib.gnuts_summary_columns(_dp(d), C, n, len(cols), n * K, K, ci, _dp(p), len(p), threads, _dp(out)))
    return [_summary_dict(o, probs) for o in out]


class Diagnosis(ctypes.Structure):
    _fields_ = [("n_treedepth_max", ctypes.c_long), ("n_divergent", ctypes.c_long), ("e_bfmi", ctypes.c_double),
                ("n_low_ess", ctypes.c_int), ("n_high_rhat", ctypes.c_int), ("has_problems", ctypes.c_int)]


def diagnose(draws, names, max_depth=10, gpu=False, threads=0):
    """CmdStan diagnose checks of a [chains, draws, columns] array whose
    columns are named by `names` (Stan CSV order: the seven sampler columns,
    then the parameters).  Returns (report text, dict of the counts)."""
    lib = load()
    d = np.ascontiguousarray(draws, dtype=np.float64)
    C, n, K = d.shape
    names = list(names)
    col = lambda nm: names.index(nm) if nm in names else -1
    pcols = [i for i, nm in enumerate(names) if "__" not in nm]
    ci = np.ascontiguousarray(pcols, dtype=np.int32)
    pn = "\n".join(names[i] for i in pcols).encode()
    buf = ctypes.create_string_buffer(1 << 16 if len(pn) < 1 << 14 else 4 * len(pn) + (1 << 16))
    res = Diagnosis()
    _check(lib.gnuts_diagnose(_dp(d), C, n, n * K, K, col("treedepth__"), col("divergent__"), col("energy__"),
                              ci.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(pcols), pn, int(max_depth),
                              int(bool(gpu)), int(threads), buf, len(buf), ctypes.byref(res)))
    return buf.value.decode(), {f: getattr(res, f) for f, _ in Diagnosis._fields_}


class GnutsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gnuts error %d: %s" % (code, msg))
        self.code = code
        self.msg = msg


class SampleArgs(ctypes.Structure):
    _fields_ = [
        ("num_chains", ctypes.c_int), ("chain_id", ctypes.c_uint), ("seed", ctypes.c_uint),
        ("init_radius", ctypes.c_double), ("num_warmup", ctypes.c_int), ("num_samples", ctypes.c_int),
        ("thin", ctypes.c_int), ("save_warmup", ctypes.c_int), ("refresh", ctypes.c_int),
        ("stepsize", ctypes.c_double), ("stepsize_jitter", ctypes.c_double), ("max_depth", ctypes.c_int),
        ("delta", ctypes.c_double), ("gamma", ctypes.c_double), ("kappa", ctypes.c_double),
        ("t0", ctypes.c_double), ("init_buffer", ctypes.c_uint), ("term_buffer", ctypes.c_uint),
        ("window", ctypes.c_uint), ("precision", ctypes.c_int),
    ]


class Var(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("type", ctypes.c_int), ("ndim", ctypes.c_int),
                ("dims", ctypes.POINTER(ctypes.c_int64)), ("data", ctypes.c_void_p)]


class Output(ctypes.Structure):
    _fields_ = [("draws", ctypes.c_void_p), ("stepsize", ctypes.c_void_p), ("inv_metric", ctypes.c_void_p),
                ("warmup_seconds", ctypes.c_void_p), ("sampling_seconds", ctypes.c_void_p),
                ("n_grad", ctypes.c_void_p), ("chain_status", ctypes.c_void_p), ("n_leapfrog", ctypes.c_void_p),
                ("timing", ctypes.c_void_p), ("diagnostics", ctypes.c_void_p)]


class TrainArgs(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("batch", ctypes.c_int), ("learning_rate", ctypes.c_double),
                ("base_scale", ctypes.c_double), ("beta0", ctypes.c_double), ("anneal_fraction", ctypes.c_double),
                ("seed", ctypes.c_uint)]


class LearnedArgs(ctypes.Structure):
    _fields_ = [("layers", ctypes.c_int), ("hidden", ctypes.c_int), ("clamp", ctypes.c_double),
                ("train", TrainArgs), ("flow_warmup", ctypes.c_int), ("flow_delta", ctypes.c_double),
                ("pilot_samples", ctypes.c_int),
                ("moment_tolerance", ctypes.c_double), ("rhat_max", ctypes.c_double)]


class LearnedReport(ctypes.Structure):
    _fields_ = [("used_flow", ctypes.c_int), ("plain_ess_per_grad", ctypes.c_double),
                ("flow_ess_per_grad", ctypes.c_double), ("plain_divergence_rate", ctypes.c_double),
                ("flow_divergence_rate", ctypes.c_double), ("max_moment_z", ctypes.c_double),
                ("loss_first", ctypes.c_double), ("loss_last", ctypes.c_double),
                ("plain_seconds", ctypes.c_double), ("train_seconds", ctypes.c_double),
                ("flow_seconds", ctypes.c_double), ("final_seconds", ctypes.c_double),
                ("plain_grads", ctypes.c_int64), ("flow_grads", ctypes.c_int64), ("final_grads", ctypes.c_int64),
                ("plain_max_rhat", ctypes.c_double), ("flow_max_rhat", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


TIMING_FIELDS = ["rounds", "grad_kernel_us", "advance_kernel_us", "device_ms", "launches", "reduce_kernel_us",
                 "chains_per_cta"]


PROGRESS_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int)
INTERRUPT_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p)
DRAWS_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double))
ERR_INTERRUPTED = 7

_lib = None


def load():
    """Load libgnuts.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise GnutsError(ERR_CUDA, "libgnuts.so not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(LIB_PATH)
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
    lib.gnuts_model_create.argtypes = [ctypes.c_char_p, ctypes.POINTER(Var), ip, ctypes.c_uint,
                                       ctypes.POINTER(vp)]
    lib.gnuts_model_create_json.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint, ctypes.POINTER(vp)]
    lib.gnuts_model_destroy.argtypes = [vp]
    lib.gnuts_model_destroy.restype = None
    lib.gnuts_model_dims.argtypes = [vp, ctypes.POINTER(ip), ctypes.POINTER(ip)]
    lib.gnuts_model_name.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    lib.gnuts_model_param_name.argtypes = [vp, ip, ip, ctypes.c_char_p, ctypes.c_size_t]
    lib.gnuts_log_prob_grad.argtypes = [vp, ip, dp, ip, dp, dp]
    lib.gnuts_log_prob_grad_precision.argtypes = [vp, ip, dp, ip, ip, dp, dp]
    # device pointers (passed as integers)
    lib.gnuts_log_prob_grad_noalloc.argtypes = [vp, ip, vp, ip, vp, vp]
    lib.gnuts_unconstrain.argtypes = [vp, dp, dp]
    lib.gnuts_write_array.argtypes = [vp, ip, dp, dp]
    lib.gnuts_sample_args_default.argtypes = [ctypes.POINTER(SampleArgs)]
    lib.gnuts_sample_args_default.restype = None
    for name in ("gnuts_hmc_nuts_diag_e_adapt", "gnuts_hmc_nuts_dense_e_adapt", "gnuts_hmc_nuts_diag_e",
                 "gnuts_hmc_nuts_dense_e"):
        getattr(lib, name).argtypes = [vp, ctypes.POINTER(SampleArgs), dp, dp, ctypes.POINTER(Output),
                                       PROGRESS_FN, vp]
    for name in ("gnuts_hmc_nuts_unit_e_adapt", "gnuts_hmc_nuts_unit_e"):
        getattr(lib, name).argtypes = [vp, ctypes.POINTER(SampleArgs), dp, ctypes.POINTER(Output), PROGRESS_FN, vp]
    lib.gnuts_transition.argtypes = [vp, ip, dp, ip, dp, dp, ctypes.c_double, ip, ctypes.c_uint,
                                     ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_uint64), dp, dp]
    lib.gnuts_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    lib.gnuts_version.restype = ctypes.c_char_p
    i64 = ctypes.c_int64
    lib.gnuts_summary.argtypes = [dp, ip, ip, i64, i64, dp, ip, dp]
    lib.gnuts_summary_columns.argtypes = [dp, ip, ip, ip, i64, i64, ctypes.POINTER(ip), dp, ip, ip, dp]
    lib.gnuts_summary_columns_gpu.argtypes = [dp, ip, ip, ip, i64, i64, ctypes.POINTER(ip), dp, ip, dp]
    lib.gnuts_set_interrupt.argtypes = [INTERRUPT_FN, ctypes.c_void_p]
    lib.gnuts_set_interrupt.restype = None
    lib.gnuts_set_draw_sink.argtypes = [DRAWS_FN, ctypes.c_void_p]
    lib.gnuts_set_draw_sink.restype = None
    lib.gnuts_diagnose.argtypes = [dp, ip, ip, i64, i64, ip, ip, ip, ctypes.POINTER(ip), ip, ctypes.c_char_p, ip, ip,
                                   ip, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_void_p]
    lib.gnuts_flow_create.argtypes = [ip, ip, ip, ctypes.c_double, ctypes.POINTER(vp)]
    lib.gnuts_flow_destroy.argtypes = [vp]
    lib.gnuts_flow_destroy.restype = None
    lib.gnuts_flow_num_params.argtypes = [vp]
    lib.gnuts_flow_num_params.restype = ctypes.c_long
    lib.gnuts_flow_set_params.argtypes = [vp, dp]
    lib.gnuts_flow_get_params.argtypes = [vp, dp]
    lib.gnuts_flow_init_affine.argtypes = [vp, dp, dp, ctypes.c_uint, ctypes.c_double]
    lib.gnuts_flow_forward.argtypes = [vp, ip, dp, dp, dp]
    lib.gnuts_flow_inverse.argtypes = [vp, ip, dp, dp, dp]
    lib.gnuts_flow_log_prob_grad.argtypes = [vp, vp, ip, dp, ip, dp, dp, dp]
    lib.gnuts_flow_log_prob_grad_tc.argtypes = [vp, vp, ip, dp, dp, dp]
    lib.gnuts_flow_adam_step.argtypes = [vp, dp, ip] + [ctypes.c_double] * 4
    lib.gnuts_train_args_default.argtypes = [ctypes.POINTER(TrainArgs)]
    lib.gnuts_train_args_default.restype = None
    lib.gnuts_flow_train.argtypes = [vp, vp, ctypes.POINTER(TrainArgs), dp]
    lib.gnuts_hmc_nuts_flow_diag_e_adapt.argtypes = [vp, vp, ctypes.POINTER(SampleArgs), dp, dp,
                                                     ctypes.POINTER(Output), PROGRESS_FN, vp]
    lib.gnuts_learned_args_default.argtypes = [ctypes.POINTER(LearnedArgs)]
    lib.gnuts_learned_args_default.restype = None
    lib.gnuts_hmc_nuts_learned_diag_e_adapt.argtypes = [vp, ctypes.POINTER(SampleArgs), ctypes.POINTER(LearnedArgs),
                                                        dp, ctypes.POINTER(Output), ctypes.POINTER(LearnedReport),
                                                        PROGRESS_FN, vp]
    _lib = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def _check(rc):
    if rc != GNUTS_OK:
        lib = load()
        buf = ctypes.create_string_buffer(4096)
        lib.gnuts_last_error(buf, len(buf))
        raise GnutsError(rc, buf.value.decode(errors="replace"))


def default_args(**kw):
    a = SampleArgs()
    load().gnuts_sample_args_default(ctypes.byref(a))
    for k, v in kw.items():
        if not hasattr(a, k):
            raise TypeError("unknown sampler argument %r" % k)
        setattr(a, k, v)
    return a


class Fit:
    """Draws and adaptation results of one run (per chain)."""

    def __init__(self, columns, draws, stepsize, inv_metric, warmup_seconds, sampling_seconds, n_grad, status,
                 n_leapfrog=None, timing=None):
        self.columns = columns
        self.draws = draws                    # [chains, n_saved, 7 + num_constrained]
        self.stepsize = stepsize
        self.inv_metric = inv_metric
        self.warmup_seconds = warmup_seconds
        self.sampling_seconds = sampling_seconds
        self.n_grad = n_grad
        self.status = status
        self.n_leapfrog = n_leapfrog          # per chain, warmup + sampling
        self.timing = dict(zip(TIMING_FIELDS, timing)) if timing is not None else {}

    def column(self, name):
        return self.draws[:, :, self.columns.index(name)]


class Model:
    """A built-in model with its data, on the GPU (model_base equivalent)."""

    def __init__(self, model_id, data=None, json_text=None, seed=0):
        lib = load()
        h = ctypes.c_void_p()
        keep = []
        if json_text is not None:
            _check(lib.gnuts_model_create_json(model_id.encode(), json_text.encode(), seed, ctypes.byref(h)))
        else:
            data = data or {}
            vars_ = (Var * max(1, len(data)))()
            for i, (name, value) in enumerate(data.items()):
                arr = np.asarray(value)
                is_int = np.issubdtype(arr.dtype, np.integer) or arr.dtype == np.bool_
                # np.array keeps 0-d scalars 0-d (ascontiguousarray would make them 1-d)
                arr = np.array(arr, dtype=np.int32 if is_int else np.float64, order="C", copy=True)
                dims = (ctypes.c_int64 * max(1, arr.ndim))(*arr.shape)
                nb = name.encode()
                keep += [arr, dims, nb]
                vars_[i].name = nb
                vars_[i].type = VAR_INT if is_int else VAR_REAL
                vars_[i].ndim = arr.ndim
                vars_[i].dims = dims
                vars_[i].data = arr.ctypes.data_as(ctypes.c_void_p)
            _check(lib.gnuts_model_create(model_id.encode(), vars_, len(data), seed, ctypes.byref(h)))
        self._h = h
        self._lib = lib
        d, c = ctypes.c_int(), ctypes.c_int()
        _check(lib.gnuts_model_dims(h, ctypes.byref(d), ctypes.byref(c)))
        self.dim = d.value
        self.num_constrained = c.value
        buf = ctypes.create_string_buffer(256)
        _check(lib.gnuts_model_name(h, buf, 256))
        self.name = buf.value.decode()
        self.param_names = []
        for i in range(self.num_constrained):
            _check(lib.gnuts_model_param_name(h, i, 0, buf, 256))
            self.param_names.append(buf.value.decode())

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.gnuts_model_destroy(h)
            self._h = None

    # -- model_base surface
    def log_prob_grad(self, q, jacobian=True, precision=None):
        q = np.ascontiguousarray(np.atleast_2d(q), dtype=np.float64)
        n = q.shape[0]
        lp = np.zeros(n)
        g = np.zeros((n, self.dim))
        if precision is None:
            _check(self._lib.gnuts_log_prob_grad(self._h, n, _dp(q), int(bool(jacobian)), _dp(lp), _dp(g)))
        else:
            _check(self._lib.gnuts_log_prob_grad_precision(self._h, n, _dp(q), int(bool(jacobian)), int(precision),
                                                           _dp(lp), _dp(g)))
        return lp, g

    def unconstrain(self, constrained):
        c = np.ascontiguousarray(constrained, dtype=np.float64)
        q = np.zeros(self.dim)
        _check(self._lib.gnuts_unconstrain(self._h, _dp(c), _dp(q)))
        return q

    def write_array(self, q):
        q = np.ascontiguousarray(np.atleast_2d(q), dtype=np.float64)
        out = np.zeros((q.shape[0], self.num_constrained))
        _check(self._lib.gnuts_write_array(self._h, q.shape[0], _dp(q), _dp(out)))
        return out

    # -- services
    def _outputs(self, a, mk, n_saved):
        C, D = a.num_chains, self.dim
        ncol = 7 + self.num_constrained
        msz = D * D if mk == 1 else D
        bufs = dict(draws=np.zeros((C, n_saved, ncol)), eps=np.zeros(C), minv=np.zeros((C, msz)), tw=np.zeros(C),
                    ts=np.zeros(C), ng=np.zeros(C, dtype=np.int64), stt=np.zeros(C, dtype=np.int32),
                    nlf=np.zeros(C, dtype=np.int64), tim=np.zeros(8))
        b = bufs
        out = Output(b["draws"].ctypes.data, b["eps"].ctypes.data, b["minv"].ctypes.data, b["tw"].ctypes.data,
                     b["ts"].ctypes.data, b["ng"].ctypes.data, b["stt"].ctypes.data, b["nlf"].ctypes.data,
                     b["tim"].ctypes.data)
        return out, bufs

    def _fit(self, b, mk):
        minv = b["minv"].reshape(len(b["eps"]), self.dim, self.dim) if mk == 1 else b["minv"]
        return Fit(SAMPLER_COLUMNS + self.param_names, b["draws"], b["eps"], minv, b["tw"], b["ts"], b["ng"],
                   b["stt"], b["nlf"], b["tim"][:len(TIMING_FIELDS)])

    def sample(self, metric="diag_e", adapt=True, inits=None, inv_metric=None, progress=None, draw_sink=None,
               interrupt=None, keep_draws=True, diagnostics=False, **kw):
        """Run hmc_nuts_<metric>[_adapt]; keyword arguments are gnuts_sample_args fields.
        draw_sink(first_row, rows) receives draw rows [chains, n, columns] while
        the run proceeds (gnuts_set_draw_sink); interrupt() returning True stops
        the run (gnuts_set_interrupt); keep_draws=False leaves the Fit's draws
        empty (the sink has them); diagnostics=True also returns the
        diagnostic_file rows as fit.diagnostics [chains, n, 7 + 3 D]."""
        a = default_args(**kw)
        C, D = a.num_chains, self.dim
        mk = METRICS[metric]
        th = max(1, a.thin)  # the library rejects thin < 1 itself
        n_saved = max(0, ((a.num_warmup + th - 1) // th if a.save_warmup else 0) + (a.num_samples + th - 1) // th)
        msz = D * D if mk == 1 else D
        out, b = self._outputs(a, mk, n_saved)
        if inits is not None:
            inits = np.ascontiguousarray(np.broadcast_to(np.asarray(inits, dtype=np.float64), (C, D)))
        if inv_metric is not None:
            im = np.asarray(inv_metric, dtype=np.float64)
            im = np.ascontiguousarray(np.broadcast_to(im.reshape(-1), (C, msz)) if im.ndim <= 2 and
                                      im.size == msz else im.reshape(C, msz))
        else:
            im = None
        cb = PROGRESS_FN(progress) if progress else PROGRESS_FN()
        name = "gnuts_hmc_nuts_%s%s" % (metric, "_adapt" if adapt else "")
        fn = getattr(self._lib, name)
        ncol = 7 + self.num_constrained
        sink_cb = DRAWS_FN(lambda ctx, first, n, rows: draw_sink(
            first, np.ctypeslib.as_array(rows, shape=(C, n, ncol)).copy())) if draw_sink else DRAWS_FN()
        int_cb = INTERRUPT_FN(lambda ctx: 1 if interrupt() else 0) if interrupt else INTERRUPT_FN()
        if not keep_draws:
            out.draws = None
            b["draws"] = np.zeros((C, 0, ncol))
        diag = np.zeros((C, n_saved, 7 + 3 * D)) if diagnostics else None
        if diag is not None:
            out.diagnostics = diag.ctypes.data
        self._lib.gnuts_set_draw_sink(sink_cb, None)
        self._lib.gnuts_set_interrupt(int_cb, None)
        try:
            if mk == 2:
                rc = fn(self._h, ctypes.byref(a), _dp(inits), ctypes.byref(out), cb, None)
            else:
                rc = fn(self._h, ctypes.byref(a), _dp(inits), _dp(im), ctypes.byref(out), cb, None)
        finally:
            self._lib.gnuts_set_draw_sink(DRAWS_FN(), None)
            self._lib.gnuts_set_interrupt(INTERRUPT_FN(), None)
        _check(rc)
        fit = self._fit(b, mk)
        fit.diagnostics = diag
        return fit

    def sample_flow(self, flow, inits_z=None, inv_metric=None, **kw):
        """hmc_nuts_diag_e_adapt on z with x = flow(z); draws are reported in x."""
        a = default_args(**kw)
        C, D = a.num_chains, self.dim
        th = max(1, a.thin)
        n_saved = max(0, ((a.num_warmup + th - 1) // th if a.save_warmup else 0) + (a.num_samples + th - 1) // th)
        out, b = self._outputs(a, 0, n_saved)
        z0 = None if inits_z is None else np.ascontiguousarray(np.broadcast_to(inits_z, (C, D)), dtype=np.float64)
        im = None if inv_metric is None else np.ascontiguousarray(np.broadcast_to(inv_metric, (C, D)),
                                                                   dtype=np.float64)
        _check(self._lib.gnuts_hmc_nuts_flow_diag_e_adapt(self._h, flow._h, ctypes.byref(a), _dp(z0), _dp(im),
                                                          ctypes.byref(out), PROGRESS_FN(), None))
        return self._fit(b, 0)

    def sample_learned(self, inits=None, learned=None, **kw):
        """Learned-preconditioner NUTS (plain diag_e as fallback and judge).
        Returns (Fit of the final draws, report dict)."""
        a = default_args(**kw)
        la = learned_args(**(learned or {}))
        C, D = a.num_chains, self.dim
        th = max(1, a.thin)
        n_saved = max(0, (a.num_samples + th - 1) // th)
        out, b = self._outputs(a, 0, n_saved)
        ini = None if inits is None else np.ascontiguousarray(np.broadcast_to(inits, (C, D)), dtype=np.float64)
        rep = LearnedReport()
        _check(self._lib.gnuts_hmc_nuts_learned_diag_e_adapt(self._h, ctypes.byref(a), ctypes.byref(la), _dp(ini),
                                                             ctypes.byref(out), ctypes.byref(rep), PROGRESS_FN(),
                                                             None))
        return self._fit(b, 0), rep.as_dict()

    def transition(self, q0, p0, stepsize, inv_metric=None, metric="diag_e", max_depth=10, seed=0,
                   chain_ids=None, counters=None):
        """One NUTS transition per row of q0 with injected momenta p0."""
        q0 = np.ascontiguousarray(np.atleast_2d(q0), dtype=np.float64)
        p0 = np.ascontiguousarray(np.atleast_2d(p0), dtype=np.float64)
        n = q0.shape[0]
        mk = METRICS[metric]
        im = None if inv_metric is None else np.ascontiguousarray(inv_metric, dtype=np.float64)
        ids = np.ascontiguousarray(chain_ids if chain_ids is not None else np.arange(1, n + 1), dtype=np.uint32)
        ctr = np.ascontiguousarray(counters if counters is not None else np.zeros(n), dtype=np.uint64)
        qo = np.zeros((n, self.dim))
        st = np.zeros((n, 7))
        _check(self._lib.gnuts_transition(self._h, mk, _dp(im), n, _dp(q0), _dp(p0), float(stepsize), max_depth,
                                          seed, ids.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)),
                                          ctr.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), _dp(qo), _dp(st)))
        return qo, st, ctr


def train_args(**kw):
    ta = TrainArgs()
    load().gnuts_train_args_default(ctypes.byref(ta))
    for k, v in kw.items():
        if not hasattr(ta, k):
            raise TypeError("unknown training argument %r" % k)
        setattr(ta, k, v)
    return ta


def learned_args(train=None, **kw):
    """Learned-sampler arguments; `train` is a dict of gnuts_train_args fields."""
    la = LearnedArgs()
    load().gnuts_learned_args_default(ctypes.byref(la))
    for k, v in kw.items():
        if not hasattr(la, k) or k == "train":
            raise TypeError("unknown learned-sampler argument %r" % k)
        setattr(la, k, v)
    for k, v in (train or {}).items():
        if not hasattr(la.train, k):
            raise TypeError("unknown training argument %r" % k)
        setattr(la.train, k, v)
    return la


class Flow:
    """Affine-coupling flow on the GPU (gnuts_flow handle)."""

    def __init__(self, dim, layers=8, hidden=128, clamp=4.0):
        lib = load()
        h = ctypes.c_void_p()
        _check(lib.gnuts_flow_create(dim, layers, hidden, float(clamp), ctypes.byref(h)))
        self._h, self._lib = h, lib
        self.dim, self.layers, self.hidden, self.clamp = dim, layers, hidden, float(clamp)
        self.n_params = lib.gnuts_flow_num_params(h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.gnuts_flow_destroy(h)
            self._h = None

    def set_params(self, theta):
        t = np.ascontiguousarray(theta, dtype=np.float64)
        assert t.shape == (self.n_params,)
        _check(self._lib.gnuts_flow_set_params(self._h, _dp(t)))

    def get_params(self):
        t = np.zeros(self.n_params)
        _check(self._lib.gnuts_flow_get_params(self._h, _dp(t)))
        return t

    def init_affine(self, mean, scale, seed=0, w1_scale=0.5):
        m = np.ascontiguousarray(np.broadcast_to(mean, (self.dim,)), dtype=np.float64)
        s = np.ascontiguousarray(np.broadcast_to(scale, (self.dim,)), dtype=np.float64)
        _check(self._lib.gnuts_flow_init_affine(self._h, _dp(m), _dp(s), seed, float(w1_scale)))

    def forward(self, z):
        z = np.ascontiguousarray(np.atleast_2d(z), dtype=np.float64)
        x, ld = np.zeros_like(z), np.zeros(z.shape[0])
        _check(self._lib.gnuts_flow_forward(self._h, z.shape[0], _dp(z), _dp(x), _dp(ld)))
        return x, ld

    def inverse(self, x):
        x = np.ascontiguousarray(np.atleast_2d(x), dtype=np.float64)
        z, ld = np.zeros_like(x), np.zeros(x.shape[0])
        _check(self._lib.gnuts_flow_inverse(self._h, x.shape[0], _dp(x), _dp(z), _dp(ld)))
        return z, ld

    def log_prob_grad(self, model, z, jacobian=True, param_grad=False):
        z = np.ascontiguousarray(np.atleast_2d(z), dtype=np.float64)
        n = z.shape[0]
        lp, gz = np.zeros(n), np.zeros_like(z)
        gth = np.zeros(self.n_params) if param_grad else None
        _check(self._lib.gnuts_flow_log_prob_grad(model._h, self._h, n, _dp(z), int(bool(jacobian)), _dp(lp),
                                                  _dp(gz), _dp(gth)))
        return (lp, gz, gth) if param_grad else (lp, gz)

    def log_prob_grad_tc(self, model, z):
        """the sampler's tensor-core gradient pass at the rows of z (Jacobian on)"""
        z = np.ascontiguousarray(np.atleast_2d(z), dtype=np.float64)
        n = z.shape[0]
        lp, gz = np.zeros(n), np.zeros_like(z)
        _check(self._lib.gnuts_flow_log_prob_grad_tc(model._h, self._h, n, _dp(z), _dp(lp), _dp(gz)))
        return lp, gz

    def adam_step(self, grad, t, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        g = np.ascontiguousarray(grad, dtype=np.float64)
        _check(self._lib.gnuts_flow_adam_step(self._h, _dp(g), int(t), lr, beta1, beta2, eps))

    def train(self, model, steps, **kw):
        """Reverse-KL training (gnuts_train_args fields as keywords); returns the loss trace."""
        ta = train_args(steps=steps, **kw)
        trace = np.zeros(max(1, steps))
        _check(self._lib.gnuts_flow_train(model._h, self._h, ctypes.byref(ta), _dp(trace)))
        return trace[:steps]

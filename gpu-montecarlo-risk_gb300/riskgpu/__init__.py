"""Python binding of the riskgpu C ABI (include/riskgpu.h, include/riskgpu_plugin.h).

A thin ctypes mirror for tests and the benchmark: the engine itself is the
sm_103a shared library `_lib/libriskgpu.so`.  Loading fails loudly when the
library is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libriskgpu.so")

RG_OK = 0
RG_ERR_INVALID = -1
RG_ERR_NOT_PD = -2
RG_ERR_CUDA = -3
RG_ERR_NOMEM = -4
RG_ERR_UNSUPPORTED = -5
RG_ERR_ADMISSION = -6
RG_ERR_NO_DEVICE = -7
RG_ERR_TIMEOUT = -8
RG_ERR_BUSY = -9

RNG_PHILOX = 0
RNG_XORWOW_REF = 1
DRAWS_DAILY = 0
DRAWS_AGGREGATED = 1
PREC_FP32 = 0
PREC_BF16X3 = 1
PREC_AUTO = 2
PREC_FP16X3 = 3
INPUT_DEVICE = 0x1

# Every symbol include/riskgpu.h and include/riskgpu_plugin.h declare.
EXPORTED_SYMBOLS = [
    "rg_abi_version", "rg_status_string", "rg_last_error", "rg_device_count",
    "rg_portfolio_create", "rg_portfolio_destroy", "rg_portfolio_info_get",
    "rg_portfolio_factor", "rg_simulate", "rg_launch_counts", "rg_run",
    "rg_estimator_stats", "rg_tail_count", "rg_probe_peaks", "rg_simulate_noalloc",
    "rg_batch_create", "rg_batch_launch", "rg_batch_wait", "rg_batch_info_get", "rg_batch_tune",
    "rg_batch_destroy", "rg_server_default_config", "rg_server_create", "rg_server_register",
    "rg_server_submit", "rg_server_wait", "rg_server_stats", "rg_server_reset_stats",
    "rg_server_destroy", "rg_moments", "rg_crash_frequency",
    "get_cuda_model", "cuda_simulate",
]


class RiskGpuError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"riskgpu status {status}: {msg}")
        self.status = status


class Query(ctypes.Structure):
    _fields_ = [("n_paths", ctypes.c_int64), ("path_offset", ctypes.c_uint64),
                ("seed", ctypes.c_uint64), ("horizon", ctypes.c_int32), ("k", ctypes.c_int32),
                ("x", ctypes.c_double), ("port_threshold", ctypes.c_double),
                ("rng", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("var_level", ctypes.c_double), ("d_s_values", ctypes.c_void_p),
                ("d_port_values", ctypes.c_void_p), ("draw_mode", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class Result(ctypes.Structure):
    _fields_ = [("n_paths", ctypes.c_int64), ("crash_count", ctypes.c_int64),
                ("breach_count", ctypes.c_int64), ("p_crash", ctypes.c_double),
                ("se_crash", ctypes.c_double), ("ci_lower", ctypes.c_double),
                ("ci_upper", ctypes.c_double), ("p_breach", ctypes.c_double),
                ("se_breach", ctypes.c_double), ("var", ctypes.c_double),
                ("cvar", ctypes.c_double), ("tail_count", ctypes.c_int64),
                ("var_passes", ctypes.c_int32), ("ms_device", ctypes.c_float)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class PortfolioInfo(ctypes.Structure):
    _fields_ = [("n_assets", ctypes.c_int32), ("has_weights", ctypes.c_int32),
                ("d_L", ctypes.c_void_p), ("d_packed", ctypes.c_void_p),
                ("wsw", ctypes.c_double), ("wmu", ctypes.c_double),
                ("ms_cholesky", ctypes.c_float)]


# ---- the reference plugin API (layout of src/model_interface.h:9-36 and
# the GSL container layout the engine reads)
class GslVector(ctypes.Structure):
    _fields_ = [("size", ctypes.c_size_t), ("stride", ctypes.c_size_t),
                ("data", ctypes.POINTER(ctypes.c_double)), ("block", ctypes.c_void_p),
                ("owner", ctypes.c_int)]


class GslMatrix(ctypes.Structure):
    _fields_ = [("size1", ctypes.c_size_t), ("size2", ctypes.c_size_t), ("tda", ctypes.c_size_t),
                ("data", ctypes.POINTER(ctypes.c_double)), ("block", ctypes.c_void_p),
                ("owner", ctypes.c_int)]


class MonteCarloResult(ctypes.Structure):
    _fields_ = [("P_hat", ctypes.c_double), ("count", ctypes.c_int),
                ("S_values", ctypes.POINTER(ctypes.c_int)), ("std_error", ctypes.c_double),
                ("ci_lower", ctypes.c_double), ("ci_upper", ctypes.c_double)]


class MonteCarloParams(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double), ("N", ctypes.c_int), ("k", ctypes.c_int),
                ("mu", ctypes.POINTER(GslVector)), ("Sigma", ctypes.POINTER(GslMatrix)),
                ("M", ctypes.c_int), ("random_seed", ctypes.c_ulong)]


ModelRunFunc = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(MonteCarloParams),
                                ctypes.POINTER(MonteCarloResult))


class ModelFunctions(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("run_model", ModelRunFunc)]


class BatchItem(ctypes.Structure):
    _fields_ = [("portfolio", ctypes.c_void_p), ("query", Query)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("items", ctypes.c_int32), ("total_tiles", ctypes.c_int64), ("unit_tiles", ctypes.c_int32),
                ("ctas_per_sm", ctypes.c_int32), ("grid", ctypes.c_int32), ("graph", ctypes.c_int32),
                ("tuned", ctypes.c_int32), ("last_ms", ctypes.c_float)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_int32), ("max_batch_items", ctypes.c_int32),
                ("headroom_bytes", ctypes.c_int64), ("admission_timeout_ms", ctypes.c_double),
                ("poll_us", ctypes.c_int32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_int64), ("refused", ctypes.c_int64), ("batches", ctypes.c_int64),
                ("mean_batch_items", ctypes.c_double), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double), ("paths_per_s", ctypes.c_double)]


class Peaks(ctypes.Structure):
    _fields_ = [("fp32_tflops", ctypes.c_double), ("normals_per_s", ctypes.c_double),
                ("sm_count", ctypes.c_int32)]


_lib = None


def lib():
    """Load libriskgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"riskgpu engine library missing: {LIB_PATH} (run build())")
        L = ctypes.CDLL(LIB_PATH)
        L.rg_status_string.restype = ctypes.c_char_p
        L.rg_last_error.restype = ctypes.c_char_p
        L.rg_portfolio_create.argtypes = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32,
                                          ctypes.POINTER(ctypes.c_void_p)]
        L.rg_portfolio_destroy.argtypes = [ctypes.c_void_p]
        L.rg_portfolio_info_get.argtypes = [ctypes.c_void_p, ctypes.POINTER(PortfolioInfo)]
        L.rg_portfolio_factor.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.rg_simulate.argtypes = [ctypes.c_void_p, ctypes.POINTER(Query), ctypes.POINTER(Result),
                                  ctypes.c_void_p]
        L.rg_simulate_noalloc.argtypes = [ctypes.c_void_p, ctypes.POINTER(Query), ctypes.POINTER(Result),
                                          ctypes.c_void_p]
        L.rg_launch_counts.argtypes = [ctypes.c_void_p, ctypes.POINTER(Query), ctypes.c_void_p,
                                       ctypes.c_void_p]
        L.rg_run.argtypes = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                             ctypes.c_void_p, ctypes.POINTER(Query), ctypes.POINTER(Result)]
        L.rg_estimator_stats.argtypes = [ctypes.c_int64, ctypes.c_int64] + [ctypes.POINTER(ctypes.c_double)] * 4
        L.rg_estimator_stats.restype = None
        L.rg_tail_count.argtypes = [ctypes.c_int64, ctypes.c_double]
        L.rg_tail_count.restype = ctypes.c_int64
        L.rg_batch_create.argtypes = [ctypes.POINTER(BatchItem), ctypes.c_int32, ctypes.c_int32,
                                      ctypes.POINTER(ctypes.c_void_p)]
        L.rg_batch_launch.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.rg_batch_wait.argtypes = [ctypes.c_void_p, ctypes.POINTER(Result)]
        L.rg_batch_info_get.argtypes = [ctypes.c_void_p, ctypes.POINTER(BatchInfo)]
        L.rg_batch_tune.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.rg_batch_destroy.argtypes = [ctypes.c_void_p]
        L.rg_server_default_config.argtypes = [ctypes.POINTER(ServerConfig)]
        L.rg_server_default_config.restype = None
        L.rg_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)]
        L.rg_server_register.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]
        L.rg_server_submit.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(Query),
                                       ctypes.POINTER(ctypes.c_uint64)]
        L.rg_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(Result),
                                     ctypes.POINTER(ctypes.c_double)]
        L.rg_server_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ServerStats)]
        L.rg_server_reset_stats.argtypes = [ctypes.c_void_p]
        L.rg_server_destroy.argtypes = [ctypes.c_void_p]
        L.rg_probe_peaks.argtypes = [ctypes.POINTER(Peaks), ctypes.c_void_p]
        L.rg_moments.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int64,
                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.rg_crash_frequency.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int64,
                                         ctypes.c_double, ctypes.c_int32, ctypes.POINTER(ctypes.c_double),
                                         ctypes.c_void_p]
        L.get_cuda_model.restype = ModelFunctions
        L.cuda_simulate.argtypes = [ctypes.POINTER(MonteCarloParams), ctypes.POINTER(MonteCarloResult)]
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != RG_OK:
        raise RiskGpuError(status, lib().rg_last_error().decode(errors="replace"))


def _host(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data


def make_query(n_paths, seed, x=0.02, k=5, horizon=1, port_threshold=-0.02, rng=RNG_PHILOX,
               precision=PREC_AUTO, var_level=0.0, path_offset=0, d_s_values=None,
               d_port_values=None, draw_mode=DRAWS_DAILY) -> Query:
    return Query(int(n_paths), int(path_offset), int(seed), int(horizon), int(k), float(x),
                 float(port_threshold), int(rng), int(precision), float(var_level),
                 d_s_values, d_port_values, int(draw_mode), 0)


class Portfolio:
    """A device-resident portfolio: FP64 Cholesky factor computed on the GPU."""

    def __init__(self, mu, sigma, weights=None, device_ptrs=None):
        L = lib()
        self._h = ctypes.c_void_p()
        if device_ptrs is not None:
            n, pmu, psig, pw = device_ptrs
            st = L.rg_portfolio_create(int(n), pmu, psig, int(n), pw, INPUT_DEVICE, ctypes.byref(self._h))
            self.n = int(n)
        else:
            mu, pmu = _host(mu)
            sigma, ps = _host(sigma)
            pw = None
            if weights is not None:
                weights, pw = _host(weights)
            self.n = int(mu.shape[0])
            st = L.rg_portfolio_create(self.n, pmu, ps, int(sigma.shape[1]), pw, 0, ctypes.byref(self._h))
        check(st)

    @property
    def handle(self):
        return self._h

    def info(self) -> dict:
        inf = PortfolioInfo()
        check(lib().rg_portfolio_info_get(self._h, ctypes.byref(inf)))
        return {f: getattr(inf, f) for f, _ in inf._fields_}

    def factor(self) -> np.ndarray:
        out = np.zeros((self.n, self.n))
        check(lib().rg_portfolio_factor(self._h, out.ctypes.data))
        return out

    def simulate(self, query: Query, stream=None) -> dict:
        r = Result()
        check(lib().rg_simulate(self._h, ctypes.byref(query), ctypes.byref(r), stream))
        return r.as_dict()

    def launch_counts(self, query: Query, d_counts_ptr: int, stream=None) -> None:
        check(lib().rg_launch_counts(self._h, ctypes.byref(query), d_counts_ptr, stream))

    def close(self):
        if self._h:
            lib().rg_portfolio_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


BATCH_NO_GRAPH = 0x1


class Batch:
    """Many (Portfolio, Query) items in one persistent tensor-core launch,
    replayed from a captured CUDA graph (rg_batch_*)."""

    def __init__(self, items, flags=0):
        self._ports = [p for p, _ in items]  # keep the portfolios alive
        arr = (BatchItem * len(items))()
        for i, (p, q) in enumerate(items):
            arr[i].portfolio = p.handle
            arr[i].query = q
        self.count = len(items)
        self._h = ctypes.c_void_p()
        check(lib().rg_batch_create(arr, self.count, flags, ctypes.byref(self._h)))

    def launch(self, stream=None):
        check(lib().rg_batch_launch(self._h, stream))

    def wait(self):
        res = (Result * self.count)()
        check(lib().rg_batch_wait(self._h, res))
        return [r.as_dict() for r in res]

    def run(self, stream=None):
        self.launch(stream)
        return self.wait()

    def tune(self, stream=None):
        check(lib().rg_batch_tune(self._h, stream))

    def info(self):
        inf = BatchInfo()
        check(lib().rg_batch_info_get(self._h, ctypes.byref(inf)))
        return {f: getattr(inf, f) for f, _ in inf._fields_}

    def close(self):
        if self._h:
            lib().rg_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request loop with continuous batching (rg_server_*)."""

    def __init__(self, **cfg):
        c = ServerConfig()
        lib().rg_server_default_config(ctypes.byref(c))
        for k, v in cfg.items():
            setattr(c, k, v)
        self._h = ctypes.c_void_p()
        self._ports = {}
        check(lib().rg_server_create(ctypes.byref(c), ctypes.byref(self._h)))

    def register(self, pid, portfolio):
        self._ports[pid] = portfolio
        check(lib().rg_server_register(self._h, int(pid), portfolio.handle))

    def submit(self, pid, query) -> int:
        t = ctypes.c_uint64()
        check(lib().rg_server_submit(self._h, int(pid), ctypes.byref(query), ctypes.byref(t)))
        return t.value

    def wait(self, ticket):
        r = Result()
        lat = ctypes.c_double()
        check(lib().rg_server_wait(self._h, ticket, ctypes.byref(r), ctypes.byref(lat)))
        d = r.as_dict()
        d["latency_ms"] = lat.value
        return d

    def try_wait(self, ticket):
        """(status, result) without raising."""
        r = Result()
        lat = ctypes.c_double()
        st = lib().rg_server_wait(self._h, ticket, ctypes.byref(r), ctypes.byref(lat))
        d = r.as_dict()
        d["latency_ms"] = lat.value
        return st, d

    def stats(self):
        s = ServerStats()
        check(lib().rg_server_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def reset_stats(self):
        check(lib().rg_server_reset_stats(self._h))

    def close(self):
        if self._h:
            lib().rg_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run(mu, sigma, weights, query: Query) -> dict:
    """One-shot from host buffers (rg_run)."""
    mu, pmu = _host(mu)
    sigma, ps = _host(sigma)
    pw = None
    if weights is not None:
        weights, pw = _host(weights)
    r = Result()
    check(lib().rg_run(int(mu.shape[0]), pmu, ps, int(sigma.shape[1]), pw, ctypes.byref(query),
                       ctypes.byref(r)))
    return r.as_dict()


def probe_peaks(stream=None) -> dict:
    pk = Peaks()
    check(lib().rg_probe_peaks(ctypes.byref(pk), stream))
    return {f: getattr(pk, f) for f, _ in pk._fields_}


def moments(returns, stream=None):
    """(mu, Sigma) of a T x N daily-returns matrix on the GPU (rg_moments):
    column means and the ddof = 1 sample covariance, FP64."""
    X = np.ascontiguousarray(returns, dtype=np.float64)
    if X.ndim != 2:
        raise ValueError("returns must be a 2-D array (days x indices)")
    T, n = X.shape
    mu = np.empty(n)
    sigma = np.empty((n, n))
    check(lib().rg_moments(X.ctypes.data, T, n, n, mu.ctypes.data, sigma.ctypes.data, stream))
    return mu, sigma


def crash_frequency(returns, x, k, stream=None) -> float:
    """Fraction of days (rows) with at least k returns below -x, on the GPU
    (rg_crash_frequency)."""
    X = np.ascontiguousarray(returns, dtype=np.float64)
    if X.ndim != 2:
        raise ValueError("returns must be a 2-D array (days x indices)")
    T, n = X.shape
    out = ctypes.c_double()
    check(lib().rg_crash_frequency(X.ctypes.data, T, n, n, float(x), int(k), ctypes.byref(out), stream))
    return out.value


def shard_range(rank: int, world: int, paths_per_rank: int):
    """Path range of one rank in a weak-scaling run: rank r owns the paths
    [r * paths_per_rank, (r + 1) * paths_per_rank) (counter-based draws: no
    state moves between ranks; the only exchange is the sum of the counts)."""
    if world < 1 or not (0 <= rank < world) or paths_per_rank < 1:
        raise ValueError("bad shard")
    return rank * paths_per_rank, paths_per_rank


def estimator_stats(count, M):
    out = [ctypes.c_double() for _ in range(4)]
    lib().rg_estimator_stats(int(count), int(M), *[ctypes.byref(o) for o in out])
    return tuple(o.value for o in out)


def tail_count(M, level):
    return int(lib().rg_tail_count(int(M), float(level)))


class PluginCall:
    """Calls the drop-in model exactly as the reference host does
    (main_runner.c:168-184, 200, 232, 248, 295): GSL-layout mu and Sigma,
    MonteCarloParams, get_cuda_model().run_model, then frees S_values."""

    def __init__(self, mu, sigma):
        self.mu = np.ascontiguousarray(mu, dtype=np.float64)
        self.sigma = np.ascontiguousarray(sigma, dtype=np.float64)
        n = self.mu.shape[0]
        self.vmu = GslVector(n, 1, self.mu.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None, 0)
        self.msig = GslMatrix(n, n, n, self.sigma.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None, 0)
        self.n = n

    def run(self, M, k, x, seed, want_S=False):
        params = MonteCarloParams(float(x), self.n, int(k), ctypes.pointer(self.vmu),
                                  ctypes.pointer(self.msig), int(M), int(seed))
        res = MonteCarloResult()
        model = lib().get_cuda_model()
        status = model.run_model(ctypes.byref(params), ctypes.byref(res))
        S = None
        if status == 0 and res.S_values:
            S = np.ctypeslib.as_array(res.S_values, shape=(int(M),)).copy()
        if res.S_values:
            libc = ctypes.CDLL(None)
            libc.free.argtypes = [ctypes.c_void_p]
            libc.free(ctypes.cast(res.S_values, ctypes.c_void_p))
        out = dict(status=status, P_hat=res.P_hat, count=res.count, std_error=res.std_error,
                   ci_lower=res.ci_lower, ci_upper=res.ci_upper, name=model.name.decode())
        if want_S:
            out["S"] = S
        return out

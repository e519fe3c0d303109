"""ORACLE TEST INFRASTRUCTURE -- not the engine.

Python side of the oracle.  Only the tests, the smoke check and the CPU
baseline leg of the benchmark import this module; the engine never does.

Contents
  * ctypes bindings for the C restatement in mc_oracle.c (_build/liboracle.so)
    and for the reference's own CPU models compiled from their sources
    (_ref/libref_cpu.so, present only where the reference tree exists);
  * `crash_simulation_numpy`: numpy restatement of the reference's Python
    model src/01-python-serial/python_serial.py:11-75 (same global numpy
    generator calls, same arithmetic), used with golden vectors generated by
    importing the reference module itself;
  * FP64 closed forms: the H-day portfolio return of R = H mu + L sum(Z) is
    exactly N(H w.mu, H w^T Sigma w), so P(breach), VaR and CVaR are exact;
    for a one-factor covariance P(S >= k) is a one-dimensional integral over
    the market factor of a Poisson-binomial tail (Gauss-Hermite quadrature);
  * the empirical VaR / CVaR definition the engine implements;
  * the reference's preprocessing (preprocessing/fetch_split.py,
    preprocessing_stats.py, evaluation.py) restated in plain Python loops
    over dicts and lists: date alignment and split, two-pass column means and
    ddof = 1 covariance, realised crash frequency.  Parity unpinned against
    the reference's own output: its pandas code cannot run here (pandas is
    not installed); these follow the documented definitions of
    DataFrame.mean / DataFrame.cov and the reference's expressions.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libref_cpu.so")
CURAND_LIB_PATH = os.path.join(HERE, "_build", "liborc_curand.so")
REF_KERNEL_PATH = os.path.join(HERE, "_ref", "ref_kernel.fatbin")

_lib = None
_ref = None
_curand = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_i64p = ctypes.POINTER(ctypes.c_longlong)


class OrcResult(ctypes.Structure):
    _fields_ = [("count", ctypes.c_longlong), ("P_hat", ctypes.c_double),
                ("std_error", ctypes.c_double), ("ci_lower", ctypes.c_double),
                ("ci_upper", ctypes.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


def build(ref: bool = False, gpu: bool = False) -> None:
    """Compile the oracle; ref=True adds the reference's CPU models (needs the
    reference tree), gpu=True the cuRAND draw helper (needs nvcc)."""
    targets = ["all"] + (["ref"] if ref else []) + (["gpu"] if gpu else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_serial_estimate.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_longlong, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_ulong, ctypes.c_int, _ip,
                                          ctypes.POINTER(OrcResult)]
        L.orc_omp_estimate.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_longlong, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_ulong, ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(OrcResult)]
        L.orc_kernel_from_normals.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_longlong, _dp,
                                              ctypes.c_double, ctypes.c_int, _ip, _dp]
        L.orc_kernel_from_normals.restype = ctypes.c_longlong
        L.orc_philox4x32_10.argtypes = [_u32p, _u32p, _u32p]
        L.orc_philox_normals.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                                         ctypes.c_int, _dp]
        L.orc_mc_philox.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, ctypes.c_longlong,
                                    ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double, ctypes.c_int,
                                    ctypes.c_double, _ip, _dp, _dp, _i64p, ctypes.c_int, ctypes.c_int]
        L.orc_cholesky_lower.argtypes = [ctypes.c_int, _dp, ctypes.c_longlong, _dp]
        L.orc_cholesky_lower.restype = ctypes.c_int
        L.orc_stats.argtypes = [ctypes.c_longlong, ctypes.c_longlong, ctypes.POINTER(OrcResult)]
        L.orc_factor_crash_prob.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp,
                                            ctypes.c_double, ctypes.c_int, ctypes.c_longlong, _dp,
                                            ctypes.c_int]
        L.orc_factor_crash_prob.restype = ctypes.c_double
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        R = ctypes.CDLL(REF_LIB_PATH)
        R.ref_run.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_int, ctypes.c_int,
                              ctypes.c_double, ctypes.c_ulong, ctypes.c_int, _ip, _dp]
        R.ref_run.restype = ctypes.c_int
        R.ref_set_threads.argtypes = [ctypes.c_int]
        _ref = R
    return _ref


def curand_lib():
    """cuRAND draw helper (GPU): the reference kernel's XORWOW normals and raw
    Philox4_32_10 words, made by calling cuRAND's device API."""
    global _curand
    if _curand is None:
        if not os.path.exists(CURAND_LIB_PATH):
            build(gpu=True)
        C = ctypes.CDLL(CURAND_LIB_PATH)
        C.orc_xorwow_normals.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.c_longlong,
                                         ctypes.c_int, _dp]
        C.orc_curand_philox_words.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong,
                                              ctypes.c_longlong, ctypes.c_int, _u32p]
        C.orc_ref_kernel_load.argtypes = [ctypes.c_char_p]
        C.orc_ref_kernel_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_ulong, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]
        _curand = C
    return _curand


def curand_xorwow_normals(seed, M, n_per_path, path0=0):
    out = np.zeros((M, n_per_path))
    if curand_lib().orc_xorwow_normals(seed, path0, M, n_per_path, out.ctypes.data_as(_dp)) != 0:
        raise RuntimeError("cuRAND XORWOW helper failed")
    return out


def curand_philox_words(seed, M, blocks, path0=0):
    out = np.zeros((M, blocks, 4), dtype=np.uint32)
    if curand_lib().orc_curand_philox_words(seed, path0, M, blocks, out.ctypes.data_as(_u32p)) != 0:
        raise RuntimeError("cuRAND Philox helper failed")
    return out


def ref_kernel_available() -> bool:
    """True where the reference's own GPU kernel has been compiled (make
    refcuda, which needs the reference tree)."""
    return os.path.exists(REF_KERNEL_PATH)


def ref_kernel_run(M, N, k, x, d_mu, d_L, seed, d_S, d_count, stream=None):
    """One launch of the reference's monte_carlo_kernel
    (src/05-GPU/monte_carlos_cuda.cu:23-72) as its host wrapper launches it
    (.cu:121-128), on device buffers given as integer addresses; returns the
    launch's device time in ms."""
    C = curand_lib()
    if C.orc_ref_kernel_load(REF_KERNEL_PATH.encode()) != 0:
        raise RuntimeError("cannot load the reference kernel from " + REF_KERNEL_PATH)
    ms = ctypes.c_float()
    if C.orc_ref_kernel_run(int(M), int(N), int(k), float(x), d_mu, d_L, int(seed), d_S, d_count, stream,
                            ctypes.byref(ms)) != 0:
        raise RuntimeError("reference kernel launch failed")
    return ms.value


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


# ---------------------------------------------------------------- C oracle
def serial_estimate(mu, sigma, M, k, x, seed, keep_upper=True, return_S=False):
    n = len(mu)
    mu, pmu = _d(mu)
    sigma, ps = _d(sigma)
    S = np.zeros(M, dtype=np.int32) if return_S else None
    res = OrcResult()
    st = lib().orc_serial_estimate(n, pmu, ps, M, k, x, seed, int(keep_upper),
                                   S.ctypes.data_as(_ip) if return_S else None, ctypes.byref(res))
    if st != 0:
        raise ValueError("oracle: Cholesky failed")
    return (res.as_dict(), S) if return_S else res.as_dict()


def omp_estimate(mu, sigma, M, k, x, seed, keep_upper=True, nthreads=0):
    n = len(mu)
    mu, pmu = _d(mu)
    sigma, ps = _d(sigma)
    res = OrcResult()
    st = lib().orc_omp_estimate(n, pmu, ps, M, k, x, seed, int(keep_upper), nthreads,
                                ctypes.byref(res))
    if st != 0:
        raise ValueError("oracle: Cholesky failed")
    return res.as_dict()


def ref_run(model, mu, sigma, M, k, x, seed, keep_upper=True, return_S=False, nthreads=0):
    """Run the reference's own serial (model='serial') or OpenMP model."""
    n = len(mu)
    if nthreads > 0:
        ref_lib().ref_set_threads(int(nthreads))
    mu, pmu = _d(mu)
    sigma, ps = _d(sigma)
    S = np.zeros(M, dtype=np.int32) if return_S else None
    out = np.zeros(6)
    ref_lib().ref_run(0 if model == "serial" else 1, n, pmu, ps, M, k, x, seed, int(keep_upper),
                      S.ctypes.data_as(_ip) if return_S else None, out.ctypes.data_as(_dp))
    res = dict(P_hat=out[0], count=int(out[1]), std_error=out[2], ci_lower=out[3],
               ci_upper=out[4], status=int(out[5]))
    return (res, S) if return_S else res


def stats(count, M):
    r = OrcResult()
    lib().orc_stats(count, M, ctypes.byref(r))
    return r.as_dict()


def cholesky_lower(A):
    A, pa = _d(A)
    n = A.shape[0]
    L = np.zeros((n, n))
    info = lib().orc_cholesky_lower(n, pa, n, L.ctypes.data_as(_dp))
    return L, info


def kernel_from_normals(mu, L, Z, x, k, return_R=False):
    """Reference GPU kernel arithmetic (FP64, fused multiply-add order)."""
    n = len(mu)
    mu, pmu = _d(mu)
    L, pL = _d(L)
    Z, pZ = _d(Z)
    M = Z.shape[0]
    S = np.zeros(M, dtype=np.int32)
    R = np.zeros((M, n)) if return_R else None
    count = lib().orc_kernel_from_normals(n, pmu, pL, M, pZ, x, k, S.ctypes.data_as(_ip),
                                          R.ctypes.data_as(_dp) if return_R else None)
    return (int(count), S, R) if return_R else (int(count), S)


def philox4x32_10(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    kk = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(c.ctypes.data_as(_u32p), kk.ctypes.data_as(_u32p),
                            out.ctypes.data_as(_u32p))
    return out


def philox_normals(seed, path, n, n_days=1):
    out = np.zeros((n_days, n))
    lib().orc_philox_normals(seed, path, n, n_days, out.ctypes.data_as(_dp))
    return out


def mc_philox(mu, L, w, n_days, M, seed, x, k, port_threshold, path_offset=0,
              want_S=False, want_port=False, want_R=False, nthreads=0, aggregated=False):
    """FP64 Monte Carlo in the engine's sampling layout (per-path parity)."""
    n = len(mu)
    mu, pmu = _d(mu)
    L, pL = _d(L)
    pw = None
    if w is not None:
        w, pw = _d(w)
    S = np.zeros(M, dtype=np.int32) if want_S else None
    port = np.zeros(M) if want_port else None
    R = np.zeros((M, n)) if want_R else None
    counts = np.zeros(2, dtype=np.int64)
    lib().orc_mc_philox(n, pmu, pL, pw, n_days, M, path_offset, seed, x, k, port_threshold,
                        S.ctypes.data_as(_ip) if want_S else None,
                        port.ctypes.data_as(_dp) if want_port else None,
                        R.ctypes.data_as(_dp) if want_R else None,
                        counts.ctypes.data_as(_i64p), nthreads, int(aggregated))
    return dict(crash=int(counts[0]), breach=int(counts[1]), S=S, port=port, R=R)


# --------------------------------------------------- numpy restatement
def crash_simulation_numpy(x, N, k, mu, Sigma, M):
    """Restatement of python_serial.py:11-75: per trial draw N standard
    normals from numpy's global generator, R = mu + L Z with numpy's
    Cholesky factor, S = #{R < -x}, count S >= k."""
    L = np.linalg.cholesky(Sigma)
    count = 0
    S_values = np.zeros(M)
    for j in range(M):
        Z = np.random.standard_normal(N)
        R = mu + L @ Z
        S = int(np.sum(R < -x))
        S_values[j] = S
        if S >= k:
            count += 1
    return count / M, count, S_values


# --------------------------------------------------------- closed forms
def _phi(z):
    return math.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def _Phi(z):
    return 0.5 * math.erfc(-z / math.sqrt(2.0))


def portfolio_closed_form(mu, sigma, w, horizon, threshold, alpha):
    """Exact H-day portfolio return distribution N(m, s^2) and its tail:
    P(w.R < threshold), VaR_alpha and CVaR_alpha of the loss -w.R."""
    from scipy.stats import norm
    w = np.asarray(w, dtype=np.float64)
    m = horizon * float(w @ mu)
    s = math.sqrt(horizon * float(w @ sigma @ w))
    p = float(norm.cdf((threshold - m) / s))
    z = float(norm.ppf(alpha))
    var = -m + s * z
    cvar = -m + s * _phi(z) / (1.0 - alpha)
    return dict(mean=m, sd=s, p_breach=p, var=var, cvar=cvar)


def one_factor_crash_prob(mu, beta, market_vol, idio, x, k, horizon=1, nodes=96):
    """P(S >= k) for R_i = H mu_i + sqrt(H)(market_vol beta_i F + idio_i e_i),
    F, e_i iid N(0,1): condition on F, the crashes are independent with
    p_i(F) = Phi((-x - H mu_i - sqrt(H) market_vol beta_i F)/(sqrt(H) idio_i));
    the conditional tail is a Poisson-binomial sum, integrated over F with
    Gauss-Hermite quadrature."""
    from scipy.special import ndtr
    t, wt = np.polynomial.hermite_e.hermegauss(nodes)  # weight exp(-t^2/2)
    wt = wt / math.sqrt(2.0 * math.pi)
    mu = np.asarray(mu)
    beta = np.asarray(beta)
    idio = np.asarray(idio)
    sh = math.sqrt(horizon)
    total = 0.0
    for f, a in zip(t, wt):
        p = ndtr((-x - horizon * mu - sh * market_vol * beta * f) / (sh * idio))
        dist = np.zeros(len(mu) + 1)
        dist[0] = 1.0
        for pi in p:
            dist[1:] = dist[1:] * (1 - pi) + dist[:-1] * pi
            dist[0] *= (1 - pi)
        total += a * dist[k:].sum()
    return float(total)


def factor_crash_prob(mu, B, idio, x, k, horizon=1, log2_points=20, scrambles=8, nthreads=0, seed=0):
    """FP64 P(S >= k) for Sigma = B B^T + diag(idio^2) (B is N x F) over an
    H-day horizon with summed daily draws (mc_oracle.c:
    orc_factor_crash_prob): the factor-conditional Poisson-binomial tail
    averaged over F ~ N(0, I_F) by randomised quasi-Monte Carlo -- `scrambles`
    independently scrambled Sobol' sets of 2^log2_points points each, mapped
    to normals by the inverse CDF.  Returns (estimate, standard error), the
    error from the spread of the independent scrambles."""
    from scipy.stats import norm, qmc
    mu = np.ascontiguousarray(mu, dtype=np.float64)
    B = np.ascontiguousarray(np.atleast_2d(np.asarray(B, dtype=np.float64).T).T)
    idio = np.ascontiguousarray(idio, dtype=np.float64)
    n, nf = B.shape
    (mu, pmu), (B, pB), (idio, pid) = _d(mu), _d(B), _d(idio)
    est = []
    for r in range(scrambles):
        U = qmc.Sobol(nf, scramble=True, seed=seed + r).random_base2(log2_points)
        F, pF = _d(norm.ppf(U))
        est.append(lib().orc_factor_crash_prob(n, nf, int(horizon), pmu, pB, pid, float(x),
                                                int(k), F.shape[0], pF, int(nthreads)))
    est = np.array(est)
    se = float(est.std(ddof=1) / math.sqrt(len(est))) if len(est) > 1 else float("nan")
    return float(est.mean()), se


# ---------------------------------------------------- empirical tail
def tail_count(M, alpha):
    """Number of paths in the (1-alpha) tail: ceil((1-alpha) M), guarded
    against binary rounding of alpha, clamped to [1, M]."""
    t = math.ceil((1.0 - alpha) * M - 1e-9)
    return int(min(max(t, 1), M))


def var_cvar(port_returns, alpha):
    """Empirical VaR / CVaR of the loss l = -w.R as the engine defines them:
    with T = tail_count(M, alpha), VaR is the T-th largest loss and CVaR the
    mean of the T largest losses."""
    loss = -np.asarray(port_returns, dtype=np.float64)
    M = loss.size
    T = tail_count(M, alpha)
    part = np.partition(loss, M - T)
    tail = part[M - T:]
    return float(tail.min()), float(tail.mean()), T


# ---------------------------------------------------------------- preprocessing
def align_and_split(series, start, end, train_ratio):
    """fetch_split.py:86-124 in plain Python: series maps name -> list of
    (date, return) with datetime.date keys; returns (train_rows, test_rows),
    each a list of (date, [returns in name order]).  Union of dates
    ascending, [start, end] inclusive, rows with a missing (None / NaN)
    return dropped, split at int(rows * train_ratio)."""
    names = list(series.keys())
    table = {}
    for j, name in enumerate(names):
        for d, r in series[name]:
            table.setdefault(d, [None] * len(names))[j] = r
    rows = []
    for d in sorted(table):
        if d < start or d > end:
            continue
        vals = table[d]
        if any(v is None or v != v for v in vals):
            continue
        rows.append((d, vals))
    split = int(len(rows) * train_ratio)
    return rows[:split], rows[split:]


def compute_stats(X):
    """preprocessing_stats.py:18,21: column means and the ddof = 1 sample
    covariance (two passes: means, then the sum of products of deviations),
    in FP64; the means with math.fsum (correctly rounded)."""
    X = np.asarray(X, dtype=np.float64)
    T, n = X.shape
    mu = np.array([math.fsum(X[:, j]) / T for j in range(n)])
    D = X - mu
    sigma = (D.T @ D) / (T - 1)
    return mu, 0.5 * (sigma + sigma.T)


def compute_metrics(X, x, k):
    """evaluation.py:19,22: fraction of rows with at least k entries < -x."""
    X = np.asarray(X, dtype=np.float64)
    days = 0
    for row in X:
        if sum(1 for v in row if v < -x) >= k:
            days += 1
    return days / len(X)

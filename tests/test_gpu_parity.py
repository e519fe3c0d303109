"""GPU parity: the engine's sm_103a kernels against the oracle, through the C ABI.

Tolerances (FP32 engine vs FP64 oracle):
  * crash count S per path: bit-exact, except paths where some asset return
    lies within NEAR = 2e-6 of the threshold (|R_i + x| < NEAR in the
    oracle's FP64 value); the number of such paths is reported and small;
  * portfolio return per path: |w.R_gpu - w.R_oracle| <= 2e-5;
  * Cholesky factor: max |L_gpu - L_oracle| <= 1e-12 (both FP64);
  * estimates vs FP64 closed forms / oracle MC: within 3 standard errors.
"""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NEAR = 2e-6
PORT_TOL = 2e-5


def _torch():
    import torch
    return torch


def _run_paths(engine, port, n_paths, seed, x, k, thr, horizon=1, rng=0, path_offset=0):
    torch = _torch()
    S = torch.full((n_paths,), -1, dtype=torch.int32, device="cuda")
    W = torch.full((n_paths,), float("nan"), dtype=torch.float32, device="cuda")
    q = engine.make_query(n_paths, seed, x=x, k=k, horizon=horizon, port_threshold=thr, rng=rng,
                          path_offset=path_offset, d_s_values=S.data_ptr(), d_port_values=W.data_ptr())
    res = port.simulate(q)
    torch.cuda.synchronize()
    return res, S.cpu().numpy(), W.cpu().numpy()


def _assert_S_parity(S_gpu, S_ref, R_ref, x, max_near_frac=1e-2):
    near = np.min(np.abs(R_ref + x), axis=1) < NEAR
    bad = (S_gpu != S_ref) & ~near
    assert not bad.any(), f"{int(bad.sum())} paths differ away from the threshold"
    assert near.mean() <= max_near_frac, near.mean()
    return int(near.sum())


@pytest.mark.parametrize("form,n", [("auto", n) for n in (1, 3, 16, 20, 33, 50, 63, 64, 65, 130, 600)]
                         + [("blocked", n) for n in (1, 3, 31, 32, 33, 64)] + [("single", 130)])
def test_cholesky_matches_oracle(gpu, oracle, monkeypatch, form, n):
    """Single-CTA form up to N = 64, blocked multi-SM form above (and either
    forced by RG_CHOLESKY): L within 1e-12 of the oracle, moments exact to
    rounding."""
    if form != "auto":
        monkeypatch.setenv("RG_CHOLESKY", form)
    from riskgpu import synth
    rng = np.random.default_rng(n)
    mu, sigma, _, _ = synth.one_factor_sigma(rng, n)
    port = gpu.Portfolio(mu, sigma, np.full(n, 1.0 / n))
    L = port.factor()
    L_ref, info = oracle.cholesky_lower(sigma)
    assert info == 0
    assert np.max(np.abs(L - L_ref)) <= 1e-12
    inf = port.info()
    w = np.full(n, 1.0 / n)
    assert abs(inf["wsw"] - w @ sigma @ w) <= 1e-15 + 1e-12 * abs(w @ sigma @ w)
    assert abs(inf["wmu"] - w @ mu) <= 1e-15


@pytest.mark.parametrize("form", ["single", "blocked"])
def test_cholesky_errors_at_a_later_pivot(gpu, monkeypatch, form):
    """A matrix that fails at column 70 (inside the third block of the
    blocked form), and a NaN in the lower triangle, give the same errors in
    both forms."""
    monkeypatch.setenv("RG_CHOLESKY", form)
    n = 100
    a = np.eye(n) * 2.0
    a[70, 70] = -1.0
    with pytest.raises(gpu.RiskGpuError) as e:
        gpu.Portfolio(np.zeros(n), a)
    assert e.value.status == gpu.RG_ERR_NOT_PD
    assert "pivot 70" in str(e.value)
    a = np.eye(n)
    a[80, 3] = np.nan
    with pytest.raises(gpu.RiskGpuError) as e:
        gpu.Portfolio(np.zeros(n), a)
    assert e.value.status == gpu.RG_ERR_INVALID


def test_cholesky_errors(gpu):
    bad = np.array([[1.0, 2.0], [2.0, 1.0]])
    with pytest.raises(gpu.RiskGpuError) as e:
        gpu.Portfolio(np.zeros(2), bad)
    assert e.value.status == gpu.RG_ERR_NOT_PD
    with pytest.raises(gpu.RiskGpuError) as e:
        gpu.Portfolio(np.zeros(2), -np.eye(2))
    assert e.value.status == gpu.RG_ERR_NOT_PD


@pytest.mark.parametrize("kernel", ["fused", "smem"])
@pytest.mark.parametrize("n,horizon,M", [(20, 1, 60000), (50, 1, 40000), (13, 4, 30000),
                                         (64, 2, 20000), (1, 1, 5000), (33, 1, 777),
                                         (57, 1, 10000), (41, 3, 9000)])
def test_philox_per_path_parity(gpu, oracle, monkeypatch, kernel, n, horizon, M):
    """Engine Philox path == oracle FP64 restatement of the same counter
    layout, per path (S exact away from the threshold, w.R within tolerance),
    for both the outer-product kernel and the row-order shared-memory one."""
    if kernel == "smem":
        monkeypatch.setenv("RG_PLAIN_KERNEL", "smem")
    else:
        monkeypatch.delenv("RG_PLAIN_KERNEL", raising=False)
    from riskgpu import synth
    rng = np.random.default_rng(100 + n)
    mu, sigma, _, _ = synth.one_factor_sigma(rng, n)
    w = rng.dirichlet(np.ones(n))
    x, k, thr, seed = 0.02 * math.sqrt(horizon), max(1, n // 4), -0.02, 1234 + n
    port = gpu.Portfolio(mu, sigma, w)
    res, S, W = _run_paths(gpu, port, M, seed, x, k, thr, horizon=horizon)
    L_ref, _ = oracle.cholesky_lower(sigma)
    ref = oracle.mc_philox(mu, L_ref, w, horizon, M, seed, x, k, thr, want_S=True, want_port=True,
                           want_R=True)
    _assert_S_parity(S, ref["S"], ref["R"], x)
    assert np.max(np.abs(W - ref["port"])) <= PORT_TOL
    assert res["crash_count"] == int((S >= k).sum())
    assert res["breach_count"] == int((W < thr).sum())
    # counts differ from the oracle's only through near-threshold paths
    near_port = np.abs(ref["port"] - thr) < PORT_TOL
    assert abs(res["breach_count"] - ref["breach"]) <= int(near_port.sum())


def test_philox_stream_is_curand_philox_layout(gpu, oracle):
    """The engine's counter layout (key = seed, counter = (block, 0, path))
    is cuRAND's curand_init(seed, path, 0) Philox4_32_10 stream: the oracle's
    Philox (pinned by the Random123 vectors) equals cuRAND's words."""
    seed, M, blocks = 0x1234_5678_9ABC, 64, 5
    words = oracle.curand_philox_words(seed, M, blocks, path0=1000)
    key = [seed & 0xFFFFFFFF, seed >> 32]
    for p in (0, 1, 17, 63):
        path = 1000 + p
        for b in range(blocks):
            ours = oracle.philox4x32_10([b, 0, path & 0xFFFFFFFF, path >> 32], key)
            assert list(ours) == list(words[p, b])


@pytest.mark.parametrize("n,M,seed", [(20, 20000, 42), (50, 20000, 67), (9, 10000, 67)])
def test_xorwow_reference_layout_parity(gpu, oracle, n, M, seed):
    """RG_RNG_XORWOW_REF reproduces the reference kernel: its normals are
    cuRAND's (curand_init(seed, path, 0) + curand_normal_double), and S per
    path equals the reference kernel's FP64 arithmetic except within NEAR of
    the threshold."""
    from riskgpu import synth
    rng = np.random.default_rng(n)
    mu, sigma, _, _ = synth.one_factor_sigma(rng, n)
    x, k = 0.02, max(1, n // 4)
    port = gpu.Portfolio(mu, sigma)
    res, S, _ = _run_paths(gpu, port, M, seed, x, k, -1.0, rng=gpu.RNG_XORWOW_REF)
    Z = oracle.curand_xorwow_normals(seed, M, n)
    L_ref, _ = oracle.cholesky_lower(sigma)
    count, S_ref, R_ref = oracle.kernel_from_normals(mu, L_ref, Z, x, k, return_R=True)
    nnear = _assert_S_parity(S, S_ref, R_ref, x)
    near_paths = np.min(np.abs(R_ref + x), axis=1) < NEAR
    assert abs(res["crash_count"] - count) <= nnear
    assert res["crash_count"] == int((S >= k).sum())
    # counts away from the threshold are identical
    assert int(((S >= k) & ~near_paths).sum()) == int(((S_ref >= k) & ~near_paths).sum())


def test_statistics_vs_closed_forms(gpu, oracle):
    """One-factor 20-asset portfolio, 2e7 paths: crash probability vs the
    Gauss-Hermite x Poisson-binomial closed form, breach probability vs the
    Gaussian closed form, both within 3 SE."""
    from riskgpu import synth
    p = synth.one_factor_20()
    rng = np.random.default_rng(42)
    mu, sigma, beta, idio = synth.one_factor_sigma(rng, 20)
    port = gpu.Portfolio(p.mu, p.sigma, p.weights)
    M = 20_000_000
    r = port.simulate(gpu.make_query(M, 42, x=p.x, k=p.k, port_threshold=p.port_threshold))
    exact = oracle.one_factor_crash_prob(mu, beta, 0.012, idio, p.x, p.k)
    assert abs(r["p_crash"] - exact) < 3 * math.sqrt(exact * (1 - exact) / M)
    cf = oracle.portfolio_closed_form(p.mu, p.sigma, p.weights, 1, p.port_threshold, 0.99)
    assert abs(r["p_breach"] - cf["p_breach"]) < 3 * math.sqrt(cf["p_breach"] * (1 - cf["p_breach"]) / M)


def test_agrees_with_reference_serial_estimator(gpu, oracle):
    """All forms agree with the reference's serial C estimator (oracle
    restatement, pure-L factor) within 3 SE of the difference."""
    from riskgpu import synth
    p = synth.one_factor_20()
    M_cpu, M_gpu = 400_000, 4_000_000
    cpu = oracle.serial_estimate(p.mu, p.sigma, M_cpu, p.k, p.x, 42, keep_upper=False)
    port = gpu.Portfolio(p.mu, p.sigma)
    for rng_layout in (gpu.RNG_PHILOX, gpu.RNG_XORWOW_REF):
        r = port.simulate(gpu.make_query(M_gpu, 42, x=p.x, k=p.k, rng=rng_layout))
        se = math.sqrt(cpu["std_error"] ** 2 + r["se_crash"] ** 2)
        assert abs(r["p_crash"] - cpu["P_hat"]) < 3 * se


def test_path_ranges_are_additive(gpu):
    """Counter-based draws: the count over [0, M) is the sum over any split
    into ranges (restartable and shardable by path offset)."""
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=1)
    port = gpu.Portfolio(p.mu, p.sigma, p.weights)
    M = 3_000_001
    full = port.simulate(gpu.make_query(M, 67, x=p.x, k=p.k, port_threshold=p.port_threshold))
    a = port.simulate(gpu.make_query(1_000_003, 67, x=p.x, k=p.k, port_threshold=p.port_threshold))
    b = port.simulate(gpu.make_query(M - 1_000_003, 67, x=p.x, k=p.k, port_threshold=p.port_threshold,
                                     path_offset=1_000_003))
    assert a["crash_count"] + b["crash_count"] == full["crash_count"]
    assert a["breach_count"] + b["breach_count"] == full["breach_count"]


def test_deterministic_repeat(gpu):
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=1)
    port = gpu.Portfolio(p.mu, p.sigma, p.weights)
    q = gpu.make_query(2_000_000, 5, x=p.x, k=p.k, port_threshold=p.port_threshold)
    a = port.simulate(q)
    b = port.simulate(q)
    assert (a["crash_count"], a["breach_count"]) == (b["crash_count"], b["breach_count"])


def test_plugin_drop_in(gpu, oracle, monkeypatch):
    """get_cuda_model().run_model through the reference plugin structures:
    status, count and statistics, S_values only on request, and the
    reference's XORWOW stream on request."""
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=1)
    call = gpu.PluginCall(p.mu, p.sigma)
    monkeypatch.delenv("RG_MATERIALIZE_S", raising=False)
    monkeypatch.delenv("RG_RNG", raising=False)
    r = call.run(100_000, p.k, p.x, 67, want_S=True)
    assert r["status"] == 0 and r["S"] is None and r["name"] == "cuda"
    direct = gpu.run(p.mu, p.sigma, None, gpu.make_query(100_000, 67, x=p.x, k=p.k))
    assert r["count"] == direct["crash_count"]
    assert r["P_hat"] == direct["p_crash"] and r["std_error"] == direct["se_crash"]
    monkeypatch.setenv("RG_MATERIALIZE_S", "1")
    monkeypatch.setenv("RG_RNG", "xorwow")
    M = 5000
    r = call.run(M, p.k, p.x, 67, want_S=True)
    assert r["status"] == 0 and r["S"] is not None
    Z = oracle.curand_xorwow_normals(67, M, p.n)
    L_ref, _ = oracle.cholesky_lower(p.sigma)
    count, S_ref, R_ref = oracle.kernel_from_normals(p.mu, L_ref, Z, p.x, p.k, return_R=True)
    _assert_S_parity(r["S"], S_ref, R_ref, p.x)
    assert r["count"] == int((r["S"] >= p.k).sum())


def test_plugin_cache_of_resident_factors(gpu, monkeypatch):
    """run_model keeps recent factors resident: a repeated call gives the
    same counts as a call that uploads and factors anew (RG_PLUGIN_CACHE=0);
    a Sigma changed in place is refactored, not served from the cache; more
    distinct inputs than cache entries still give the right counts."""
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=1)
    call = gpu.PluginCall(p.mu, p.sigma)
    args = (200_000, p.k, p.x, p.seed)

    def fresh(c):
        monkeypatch.setenv("RG_PLUGIN_CACHE", "0")
        r = c.run(*args)
        monkeypatch.delenv("RG_PLUGIN_CACHE")
        return r

    ref = fresh(call)
    a, b = call.run(*args), call.run(*args)
    assert a["count"] == b["count"] == ref["count"]
    call.sigma[:, :] = call.sigma * 1.8      # same buffer, new values: more crashes
    c = call.run(*args)
    assert c["count"] == fresh(call)["count"] and c["count"] > a["count"]
    rng = np.random.default_rng(8)
    for i in range(6):
        mu, sigma, _, _ = synth.one_factor_sigma(rng, 20 + i)
        ci = gpu.PluginCall(mu, sigma)
        assert ci.run(*args)["count"] == fresh(ci)["count"]
    assert call.run(*args)["count"] == c["count"]


def test_plugin_errors(gpu):
    call = gpu.PluginCall(np.zeros(2), np.array([[1.0, 2.0], [2.0, 1.0]]))
    assert call.run(1000, 1, 0.02, 1)["status"] == -1


def test_fault_injection_and_admission(gpu, monkeypatch):
    from riskgpu import synth
    p = synth.one_factor_20(n_paths=1)
    monkeypatch.setenv("RG_FAULT_INJECT", "alloc")
    with pytest.raises(gpu.RiskGpuError) as e:
        gpu.Portfolio(p.mu, p.sigma)
    assert e.value.status == gpu.RG_ERR_NOMEM
    monkeypatch.delenv("RG_FAULT_INJECT")
    monkeypatch.setenv("RG_MEM_HEADROOM_BYTES", str(1 << 60))
    with pytest.raises(gpu.RiskGpuError) as e:
        gpu.Portfolio(p.mu, p.sigma)
    assert e.value.status == gpu.RG_ERR_ADMISSION
    monkeypatch.delenv("RG_MEM_HEADROOM_BYTES")
    port = gpu.Portfolio(p.mu, p.sigma)
    assert port.simulate(gpu.make_query(1000, 1))["n_paths"] == 1000


def test_runner_binary_end_to_end(gpu, tmp_path):
    """The C host driver loads the reference's .bin format and calls the
    drop-in model like main_runner."""
    import subprocess
    from riskgpu import synth, build
    p = synth.one_factor_50(n_paths=1)
    synth.write_reference_bins(p, str(tmp_path))
    out = subprocess.run([build.RUNNER, "-d", str(tmp_path), "-M", "200000", "-k", str(p.k), "-x",
                          str(p.x), "-s", "67"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert "cuda RESULTS" in out.stdout
    count = int(out.stdout.split("Extreme Events Count: ")[1].split()[0])
    direct = gpu.run(p.mu, p.sigma, None, gpu.make_query(200_000, 67, x=p.x, k=p.k))
    assert count == direct["crash_count"]


# ------------------------------------------------------------------ VaR / CVaR
def _var_case(gpu, n_paths, level=0.99, horizon=1, seed=11, n=50):
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=1)
    if n != 50:
        rng = np.random.default_rng(n)
        mu, sigma, _, _ = synth.one_factor_sigma(rng, n)
        w = rng.dirichlet(np.ones(n))
    else:
        mu, sigma, w = p.mu, p.sigma, p.weights
    port = gpu.Portfolio(mu, sigma, w)
    torch = _torch()
    W = torch.empty(n_paths, dtype=torch.float32, device="cuda")
    q = gpu.make_query(n_paths, seed, x=0.03, k=5, horizon=horizon, port_threshold=-0.03,
                       var_level=level, d_port_values=W.data_ptr())
    r = port.simulate(q)
    torch.cuda.synchronize()
    return r, W.cpu().numpy().astype(np.float64), (mu, sigma, w)


@pytest.mark.parametrize("M,level,horizon", [(200_000, 0.99, 1), (1_000_003, 0.975, 3), (1000, 0.99, 1),
                                             (100, 0.99, 1), (1, 0.5, 1)])
def test_var_cvar_exact_order_statistics(gpu, oracle, M, level, horizon):
    """VaR/CVaR from the fused band pass equal the order statistics of the
    engine's own per-path portfolio returns (definition of the oracle:
    T = ceil((1-level) M) largest losses; VaR the smallest of them, CVaR their
    mean)."""
    r, W, _ = _var_case(gpu, M, level, horizon)
    var, cvar, T = oracle.var_cvar(W, level)
    assert r["tail_count"] == T
    assert r["var"] == var
    assert abs(r["cvar"] - cvar) <= 1e-12 + 1e-9 * abs(cvar)
    assert r["var_passes"] == 1


def test_var_fallback_passes(gpu, oracle, monkeypatch):
    """With the predicted band displaced (host-side injection) the histogram
    pass and the bin-select pass find the same order statistics."""
    monkeypatch.setenv("RG_FAULT_INJECT", "varband")
    r, W, _ = _var_case(gpu, 300_000, 0.99)
    var, cvar, T = oracle.var_cvar(W, 0.99)
    assert r["var_passes"] == 3
    assert r["var"] == var and abs(r["cvar"] - cvar) <= 1e-9 * abs(cvar)


def test_var_matches_fp64_oracle_per_path(gpu, oracle):
    """Against the FP64 restatement of the same paths: VaR/CVaR within the
    per-path return tolerance."""
    M = 200_000
    r, W, (mu, sigma, w) = _var_case(gpu, M, 0.99, n=20)
    L_ref, _ = oracle.cholesky_lower(sigma)
    ref = oracle.mc_philox(mu, L_ref, w, 1, M, 11, 0.03, 5, -0.03, want_port=True)
    var, cvar, _ = oracle.var_cvar(ref["port"], 0.99)
    assert abs(r["var"] - var) <= PORT_TOL and abs(r["cvar"] - cvar) <= PORT_TOL


def test_var_cvar_vs_closed_form(gpu, oracle):
    """2e7 paths: VaR within 3 quantile standard errors and CVaR within 3
    of its standard error of the exact Gaussian values."""
    from scipy.stats import norm
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=1)
    port = gpu.Portfolio(p.mu, p.sigma, p.weights)
    M, a = 20_000_000, 0.99
    r = port.simulate(gpu.make_query(M, 3, x=p.x, k=p.k, port_threshold=p.port_threshold, var_level=a))
    cf = oracle.portfolio_closed_form(p.mu, p.sigma, p.weights, 1, p.port_threshold, a)
    z = norm.ppf(a)
    se_q = math.sqrt(a * (1 - a) / M) / (norm.pdf(z) / cf["sd"])
    assert abs(r["var"] - cf["var"]) < 3 * se_q
    # CVaR standard error: sd of the tail losses / sqrt(T)
    tail_sd = cf["sd"] * math.sqrt(1 + z * norm.pdf(z) / (1 - a) - (norm.pdf(z) / (1 - a)) ** 2)
    se_c = math.sqrt((tail_sd ** 2 + a * (cf["cvar"] - cf["var"]) ** 2) / ((1 - a) * M))
    assert abs(r["cvar"] - cf["cvar"]) < 3 * se_c


def test_var_requires_weights_and_philox(gpu):
    from riskgpu import synth
    p = synth.one_factor_20(n_paths=1)
    port = gpu.Portfolio(p.mu, p.sigma)
    with pytest.raises(gpu.RiskGpuError) as e:
        port.simulate(gpu.make_query(1000, 1, var_level=0.99))
    assert e.value.status == gpu.RG_ERR_INVALID
    port = gpu.Portfolio(p.mu, p.sigma, p.weights)
    with pytest.raises(gpu.RiskGpuError) as e:
        port.simulate(gpu.make_query(1000, 1, var_level=0.99, rng=gpu.RNG_XORWOW_REF))
    assert e.value.status == gpu.RG_ERR_UNSUPPORTED


def test_var_pass_does_not_change_counts(gpu):
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=1)
    port = gpu.Portfolio(p.mu, p.sigma, p.weights)
    q0 = gpu.make_query(3_000_000, 9, x=p.x, k=p.k, port_threshold=p.port_threshold)
    q1 = gpu.make_query(3_000_000, 9, x=p.x, k=p.k, port_threshold=p.port_threshold, var_level=0.99)
    a, b = port.simulate(q0), port.simulate(q1)
    assert (a["crash_count"], a["breach_count"]) == (b["crash_count"], b["breach_count"])
    c = port.simulate(q1)
    assert (b["var"], b["cvar"]) == (c["var"], c["cvar"])


# --------------------------------------------------------- general-N kernel
def _factor_case(n, seed, factors=5):
    from riskgpu import synth
    rng = np.random.default_rng(seed)
    if factors == 1:
        mu, sigma, _, _ = synth.one_factor_sigma(rng, n)
    else:
        mu, sigma, _, _ = synth.factor_sigma(rng, n, factors, 0.5 * 0.01)
    w = rng.dirichlet(np.ones(n))
    return mu, sigma, w


# the general-N FP32 kernels: pipelined (default), phase-serial and
# warp-specialised (RG_PLAIN_KERNEL=tiled, tiled-serial or tiled-ws forces
# one, also for N <= 64)
TILED_FORMS = ["pipe", "serial", "ws"]
TILED_ENV = {"pipe": "tiled", "serial": "tiled-serial", "ws": "tiled-ws"}


@pytest.mark.parametrize("form", TILED_FORMS)
@pytest.mark.parametrize("n,horizon,M", [(65, 1, 20000), (100, 3, 8000), (129, 1, 8000), (257, 1, 3001),
                                         (300, 2, 3000), (513, 1, 1000), (600, 10, 1024), (768, 1, 700),
                                         (700, 2, 33)])
def test_tiled_per_path_parity(gpu, oracle, monkeypatch, form, n, horizon, M):
    """General-N FP32 kernels == oracle FP64 restatement per path (sizes
    cover 1-3 column blocks of either width, partial last blocks and a path
    count that is not a multiple of the tile)."""
    monkeypatch.setenv("RG_PLAIN_KERNEL", TILED_ENV[form])
    mu, sigma, w = _factor_case(n, 7 + n)
    x = 0.02 * math.sqrt(horizon)
    k, thr, seed = max(1, n // 10), -0.03, 99 + n
    port = gpu.Portfolio(mu, sigma, w)
    res, S, W = _run_paths(gpu, port, M, seed, x, k, thr, horizon=horizon)
    L_ref, _ = oracle.cholesky_lower(sigma)
    ref = oracle.mc_philox(mu, L_ref, w, horizon, M, seed, x, k, thr, want_S=True, want_port=True,
                           want_R=True)
    _assert_S_parity(S, ref["S"], ref["R"], x, max_near_frac=5e-2)
    assert np.max(np.abs(W - ref["port"])) <= PORT_TOL
    assert res["crash_count"] == int((S >= k).sum())
    assert res["breach_count"] == int((W < thr).sum())


def test_tiled_agrees_with_fused_for_small_n(gpu, monkeypatch):
    """For N <= 64 the tiled kernel (forced) and the fused kernel draw the
    same normals: S equal per path away from the threshold, w.R within FP32
    tolerance."""
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=1)
    port = gpu.Portfolio(p.mu, p.sigma, p.weights)
    M = 50000
    monkeypatch.delenv("RG_PLAIN_KERNEL", raising=False)
    r1, S1, W1 = _run_paths(gpu, port, M, 4, p.x, p.k, p.port_threshold, horizon=2)
    monkeypatch.setenv("RG_PLAIN_KERNEL", "tiled")
    r2, S2, W2 = _run_paths(gpu, port, M, 4, p.x, p.k, p.port_threshold, horizon=2)
    assert np.max(np.abs(W1 - W2)) <= 1e-5
    assert (S1 != S2).mean() < 1e-3


@pytest.mark.parametrize("n", [20, 200])
def test_aggregated_draws_parity(gpu, oracle, n):
    """RG_DRAWS_AGGREGATED: one N(0,1) draw per asset times sqrt(H), per path
    against the oracle's restatement of the same mode."""
    mu, sigma, w = _factor_case(n, 3 + n, factors=1)
    H, M, seed = 10, 5000, 17
    x, k, thr = 0.06, max(1, n // 10), -0.05
    port = gpu.Portfolio(mu, sigma, w)
    torch = _torch()
    S = torch.empty(M, dtype=torch.int32, device="cuda")
    W = torch.empty(M, dtype=torch.float32, device="cuda")
    q = gpu.make_query(M, seed, x=x, k=k, horizon=H, port_threshold=thr, d_s_values=S.data_ptr(),
                       d_port_values=W.data_ptr(), draw_mode=gpu.DRAWS_AGGREGATED)
    port.simulate(q)
    torch.cuda.synchronize()
    L_ref, _ = oracle.cholesky_lower(sigma)
    ref = oracle.mc_philox(mu, L_ref, w, H, M, seed, x, k, thr, want_S=True, want_port=True, want_R=True,
                           aggregated=True)
    _assert_S_parity(S.cpu().numpy(), ref["S"], ref["R"], x, max_near_frac=5e-2)
    assert np.max(np.abs(W.cpu().numpy() - ref["port"])) <= PORT_TOL


def test_aggregated_statistics_match_daily(gpu, oracle):
    """Both draw modes sample the same N(H w.mu, H w'Sigma w): breach
    probabilities agree with the closed form within 3 SE."""
    mu, sigma, w = _factor_case(120, 5)
    port = gpu.Portfolio(mu, sigma, w)
    M, H, thr = 4_000_000, 10, -0.04
    cf = oracle.portfolio_closed_form(mu, sigma, w, H, thr, 0.99)
    se = math.sqrt(cf["p_breach"] * (1 - cf["p_breach"]) / M)
    for mode in (gpu.DRAWS_DAILY, gpu.DRAWS_AGGREGATED):
        r = port.simulate(gpu.make_query(M, 8, x=0.1, k=12, horizon=H, port_threshold=thr, draw_mode=mode))
        assert abs(r["p_breach"] - cf["p_breach"]) < 3 * se


@pytest.mark.parametrize("n,horizon", [(150, 1), (600, 10), (97, 2), (768, 1)])
def test_tiled_forms_identical_per_path(gpu, monkeypatch, n, horizon):
    """The phase-serial and warp-specialised FP32 kernels evaluate every
    asset return with the same FMA chain: S identical on every path, w.R
    within FP32 summation-order rounding, counts equal; the pipelined form
    agrees up to FP32 rounding of the sum order."""
    mu, sigma, w = _factor_case(n, 31 + n)
    port = gpu.Portfolio(mu, sigma, w)
    M, x, k, thr = 40_000, 0.02 * math.sqrt(horizon), max(1, n // 10), -0.03
    out = {}
    for form in TILED_FORMS:
        monkeypatch.setenv("RG_PLAIN_KERNEL", TILED_ENV[form])
        out[form] = _run_paths(gpu, port, M, 5, x, k, thr, horizon=horizon)
    r0, S0, W0 = out["serial"]
    r1, S1, W1 = out["ws"]
    assert (S1 == S0).all()
    assert np.max(np.abs(W1 - W0)) <= 2e-6
    assert r1["crash_count"] == r0["crash_count"]
    # the pipelined form sums the same terms in descending k: S may differ
    # only where an asset return sits within FP32 rounding of the threshold
    r2, S2, W2 = out["pipe"]
    assert (S2 != S0).mean() < 1e-3
    assert np.max(np.abs(W2 - W0)) <= 5e-6
    assert abs(r2["crash_count"] - r0["crash_count"]) <= int((S2 != S0).sum())


@pytest.mark.parametrize("form", TILED_FORMS)
def test_tiled_var_exact(gpu, oracle, monkeypatch, form):
    monkeypatch.setenv("RG_PLAIN_KERNEL", TILED_ENV[form])
    r, W, _ = _var_case(gpu, 300_000, 0.99, n=150)
    var, cvar, T = oracle.var_cvar(W, 0.99)
    assert r["var"] == var and abs(r["cvar"] - cvar) <= 1e-9 * abs(cvar)

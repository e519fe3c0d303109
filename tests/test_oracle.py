"""Oracle pins (CPU): known-answer vectors, golden vectors from the
reference's own code, closed forms.  The oracle is only trusted for the GPU
parity tests because these pass."""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN


# Random123 known-answer vectors for Philox4x32-10 (Salmon et al., SC'11;
# kat_vectors distributed with Random123): (counter, key) -> output.
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,want", PHILOX_KAT)
def test_philox_known_answers(oracle, ctr, key, want):
    assert list(oracle.philox4x32_10(ctr, key)) == want


def test_mt19937_known_answer(oracle):
    """C++ standard [rand.predef]: the 10000th output of mt19937 seeded with
    5489 is 4123659995; mt19937ar's first output for that seed is 3499211612."""
    import ctypes
    L = oracle.lib()
    L.gsl_rng_alloc.restype = ctypes.c_void_p
    L.gsl_rng_alloc.argtypes = [ctypes.c_void_p]
    L.gsl_rng_set.argtypes = [ctypes.c_void_p, ctypes.c_ulong]
    L.gsl_rng_get.argtypes = [ctypes.c_void_p]
    L.gsl_rng_get.restype = ctypes.c_ulong
    L.gsl_rng_free.argtypes = [ctypes.c_void_p]
    mt_type = ctypes.c_void_p.in_dll(L, "gsl_rng_mt19937")
    r = L.gsl_rng_alloc(mt_type.value)
    L.gsl_rng_set(r, 5489)
    first = L.gsl_rng_get(r)
    for _ in range(9998):
        L.gsl_rng_get(r)
    last = L.gsl_rng_get(r)
    L.gsl_rng_free(r)
    assert first == 3499211612
    assert last == 4123659995


def test_python_reference_golden(oracle):
    """numpy restatement == the reference's python_serial.py (imported and run
    by tests/golden/make_golden.py) per path."""
    g = np.load(os.path.join(GOLDEN, "python_serial.npz"))
    for case in ("cfg20", "example10"):
        np.random.seed(int(g[f"{case}__seed"]))
        P, count, S = oracle.crash_simulation_numpy(float(g[f"{case}__x"]), len(g[f"{case}__mu"]),
                                                    int(g[f"{case}__k"]), g[f"{case}__mu"],
                                                    g[f"{case}__sigma"], int(g[f"{case}__M"]))
        assert count == int(g[f"{case}__count"])
        assert np.array_equal(S.astype(np.int8), g[f"{case}__S"])


@pytest.mark.parametrize("keep", [1, 0])
def test_c_serial_restatement_matches_reference_golden(oracle, keep):
    """C restatement == the reference's monte_carlo_serial.c (compiled from its
    own source against the same GSL shim) per path, both factor semantics."""
    g = np.load(os.path.join(GOLDEN, "ref_c_serial.npz"))
    from riskgpu import synth
    p = synth.one_factor_20()
    assert np.array_equal(p.mu, g["mu"]) and np.array_equal(p.sigma, g["sigma"])
    r, S = oracle.serial_estimate(g["mu"], g["sigma"], int(g["M"]), int(g["k"]), float(g["x"]),
                                  int(g["seed"]), keep_upper=bool(keep), return_S=True)
    assert np.array_equal(S.astype(np.int8), g[f"serial_keep{keep}_S"])
    assert r["count"] == int(g[f"serial_keep{keep}_count"])
    np.testing.assert_allclose([r["P_hat"], r["std_error"], r["ci_lower"], r["ci_upper"]],
                               g[f"serial_keep{keep}_stats"], rtol=0, atol=0)
    # the OpenMP model draws the same set of normal vectors: same count
    assert int(g[f"openmp_keep{keep}_count"]) == r["count"]


def test_omp_restatement_count_equals_serial(oracle):
    from riskgpu import synth
    p = synth.one_factor_20()
    a = oracle.serial_estimate(p.mu, p.sigma, 20000, p.k, p.x, 42)
    b = oracle.omp_estimate(p.mu, p.sigma, 20000, p.k, p.x, 42, nthreads=4)
    assert a["count"] == b["count"]


@pytest.mark.skipif(not os.path.isdir("/root/reference/src"), reason="reference tree absent")
def test_oracle_against_live_reference(oracle):
    """Where the reference tree exists, run its C models live (not only the
    committed fixtures) on another seed and compare per path."""
    oracle.build(ref=True)
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=3000)
    import contextlib, io
    with contextlib.redirect_stdout(io.StringIO()):
        r_ref, S_ref = oracle.ref_run("serial", p.mu, p.sigma, 3000, p.k, p.x, 99, True, True)
    r, S = oracle.serial_estimate(p.mu, p.sigma, 3000, p.k, p.x, 99, True, True)
    assert np.array_equal(S, S_ref) and r["count"] == r_ref["count"]


def test_cholesky_vs_numpy(oracle):
    from riskgpu import synth
    for p in (synth.one_factor_20(), synth.one_factor_50()):
        L, info = oracle.cholesky_lower(p.sigma)
        assert info == 0
        np.testing.assert_allclose(L, np.linalg.cholesky(p.sigma), rtol=0, atol=1e-15)
    bad = np.array([[1.0, 2.0], [2.0, 1.0]])
    assert oracle.cholesky_lower(bad)[1] == 2


def test_philox_mc_matches_one_factor_closed_form(oracle):
    """FP64 MC in the engine's layout agrees with Gauss-Hermite x
    Poisson-binomial closed form within 3 SE, and the portfolio tail with the
    Gaussian closed form."""
    import math
    from riskgpu import synth
    rng = np.random.default_rng(42)
    mu, sigma, beta, idio = synth.one_factor_sigma(rng, 20)
    p = synth.one_factor_20()
    assert np.array_equal(mu, p.mu)
    M = 400_000
    L, _ = oracle.cholesky_lower(p.sigma)
    mc = oracle.mc_philox(p.mu, L, p.weights, 1, M, 42, p.x, p.k, p.port_threshold, want_port=True)
    exact = oracle.one_factor_crash_prob(mu, beta, 0.012, idio, p.x, p.k)
    se = math.sqrt(exact * (1 - exact) / M)
    assert abs(mc["crash"] / M - exact) < 3 * se
    cf = oracle.portfolio_closed_form(p.mu, p.sigma, p.weights, 1, p.port_threshold, 0.99)
    se_b = math.sqrt(cf["p_breach"] * (1 - cf["p_breach"]) / M)
    assert abs(mc["breach"] / M - cf["p_breach"]) < 3 * se_b
    var, cvar, T = oracle.var_cvar(mc["port"], 0.99)
    # quantile SE: sqrt(a(1-a)/M) / f(q)
    from scipy.stats import norm
    z = norm.ppf(0.99)
    se_q = math.sqrt(0.99 * 0.01 / M) / (norm.pdf(z) / cf["sd"])
    assert abs(var - cf["var"]) < 3 * se_q
    assert T == 4000


def test_horizon_closed_form(oracle):
    """H summed daily draws: portfolio return ~ N(H w.mu, H w'Sigma w)."""
    import math
    from riskgpu import synth
    p = synth.one_factor_20()
    M, H = 200_000, 7
    L, _ = oracle.cholesky_lower(p.sigma)
    mc = oracle.mc_philox(p.mu, L, p.weights, H, M, 5, p.x, p.k, -0.05)
    cf = oracle.portfolio_closed_form(p.mu, p.sigma, p.weights, H, -0.05, 0.99)
    se = math.sqrt(cf["p_breach"] * (1 - cf["p_breach"]) / M)
    assert abs(mc["breach"] / M - cf["p_breach"]) < 3 * se


def test_keep_upper_changes_reference_cpu_estimate(oracle):
    """The reference CPU models multiply by the whole decomp1 output, whose
    strict upper triangle still holds Sigma; with it the estimate moves."""
    from riskgpu import synth
    p = synth.one_factor_20()
    a = oracle.serial_estimate(p.mu, p.sigma, 50000, p.k, p.x, 1, keep_upper=True)
    b = oracle.serial_estimate(p.mu, p.sigma, 50000, p.k, p.x, 1, keep_upper=False)
    assert a["count"] != b["count"]


def test_tail_count_definition(oracle):
    assert oracle.tail_count(1_000_000, 0.99) == 10_000
    assert oracle.tail_count(100, 0.99) == 1
    assert oracle.tail_count(150, 0.99) == 2
    assert oracle.tail_count(1, 0.99) == 1


def test_factor_crash_prob_matches_one_factor_quadrature(oracle):
    """The multi-factor P(S >= k) oracle (factor-conditional Poisson-binomial
    tail, randomised QMC) agrees with the one-factor Gauss-Hermite closed form
    within 4 of its own standard errors, for one and ten days."""
    from riskgpu import synth
    rng = np.random.default_rng(67)
    mu, sigma, beta, idio = synth.one_factor_sigma(rng, 50)
    for horizon, x, k in ((1, 0.03, 5), (10, 0.08, 8)):
        gh = oracle.one_factor_crash_prob(mu, beta, 0.012, idio, x, k, horizon)
        est, se = oracle.factor_crash_prob(mu, 0.012 * beta, idio, x, k, horizon, log2_points=12, scrambles=8)
        assert se > 0 and abs(est - gh) <= 4 * se + 1e-12, (est, se, gh)


def test_oracle_figures_fixture_belongs_to_the_workloads(oracle):
    """tests/golden/oracle_figures.json (make_oracle_figures.py) was made from
    the benchmark's synthetic inputs: its checksum matches, its closed forms
    are recomputed, and its five-factor P(S >= k) agrees with a small fresh
    oracle run within 4 standard errors."""
    import hashlib
    import json
    from riskgpu import synth
    figs = json.load(open(os.path.join(GOLDEN, "oracle_figures.json")))
    for name, make in (("one_factor_50", synth.one_factor_50), ("five_factor_600", synth.five_factor_600)):
        p = make(n_paths=1)
        fig = figs[name]
        h = hashlib.sha256()
        for a in (p.mu, p.sigma, p.weights):
            h.update(np.ascontiguousarray(a, dtype=np.float64).tobytes())
        assert h.hexdigest() == fig["inputs_sha256"], name
        cf = oracle.portfolio_closed_form(p.mu, p.sigma, p.weights, p.horizon, p.port_threshold, figs["alpha"])
        for key in ("p_breach", "var", "cvar", "mean", "sd"):
            assert abs(cf[key] - fig[key]) <= 1e-12 * max(1.0, abs(cf[key])), (name, key)
        assert (fig["x"], fig["k"], fig["horizon"], fig["port_threshold"]) == (p.x, p.k, p.horizon,
                                                                                p.port_threshold)
    p = synth.five_factor_600(n_paths=1)
    rng = np.random.default_rng(600)
    mu, sigma, B, idio = synth.factor_sigma(rng, p.n, 5, 0.5 * 0.01)
    est, se = oracle.factor_crash_prob(mu, B, idio, p.x, p.k, p.horizon, log2_points=11, scrambles=4)
    fig = figs["five_factor_600"]
    assert abs(est - fig["p_crash"]) <= 4 * math.hypot(se, fig["p_crash_se"]), (est, se, fig["p_crash"])

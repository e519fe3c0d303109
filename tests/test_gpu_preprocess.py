"""Preprocessing on the GPU (rg_moments, rg_crash_frequency) against the
oracle's restatement of preprocessing_stats.py:18,21 and evaluation.py:19,22.

Tolerances: mu and Sigma within 1e-12 relative to the largest |entry| (FP64,
different summation orders); the crash frequency exact (an integer count)."""
import ctypes
import datetime as dt

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _returns(rng, T, n):
    # correlated daily returns with a market factor, like index returns
    f = rng.normal(0, 0.01, size=(T, 1))
    beta = rng.uniform(0.5, 1.5, size=(1, n))
    return 3e-4 + f * beta + rng.normal(0, 0.008, size=(T, n))


@pytest.mark.parametrize("T,n", [(2, 1), (3, 5), (100, 33), (257, 64), (2500, 65), (2000, 600)])
def test_moments_match_the_oracle(gpu, oracle, T, n):
    X = _returns(np.random.default_rng(T * 1000 + n), T, n)
    mu, sigma = gpu.moments(X)
    mu_ref, sigma_ref = oracle.compute_stats(X)
    assert np.max(np.abs(mu - mu_ref)) <= 1e-12 * np.max(np.abs(mu_ref))
    assert np.max(np.abs(sigma - sigma_ref)) <= 1e-12 * np.max(np.abs(sigma_ref))
    assert np.array_equal(sigma, sigma.T)
    # deterministic
    mu2, sigma2 = gpu.moments(X)
    assert np.array_equal(mu, mu2) and np.array_equal(sigma, sigma2)


def test_moments_leading_dimension(gpu, oracle):
    """Rows of a wider host array (ld > n) through the C ABI."""
    rng = np.random.default_rng(5)
    T, n, ld = 300, 40, 47
    W = _returns(rng, T, ld)
    mu = np.empty(n)
    sigma = np.empty((n, n))
    gpu.check(gpu.lib().rg_moments(W.ctypes.data, T, n, ld, mu.ctypes.data, sigma.ctypes.data, None))
    mu_ref, sigma_ref = oracle.compute_stats(W[:, :n])
    assert np.max(np.abs(sigma - sigma_ref)) <= 1e-12 * np.max(np.abs(sigma_ref))
    assert np.max(np.abs(mu - mu_ref)) <= 1e-12 * np.max(np.abs(mu_ref))


@pytest.mark.parametrize("x,k", [(0.02, 1), (0.02, 5), (0.01, 3), (0.0, 10), (0.05, 1)])
def test_crash_frequency_exact(gpu, oracle, x, k):
    X = _returns(np.random.default_rng(11), 3000, 15)
    assert gpu.crash_frequency(X, x, k) == oracle.compute_metrics(X, x, k)


def test_preprocess_rejects_bad_input(gpu):
    with pytest.raises(gpu.RiskGpuError) as e:
        gpu.moments(np.zeros((1, 3)))
    assert e.value.status == gpu.RG_ERR_INVALID
    X = np.zeros((10, 3))
    X[4, 2] = np.nan
    with pytest.raises(gpu.RiskGpuError) as e:
        gpu.moments(X)
    assert e.value.status == gpu.RG_ERR_INVALID
    with pytest.raises(gpu.RiskGpuError) as e:
        gpu.crash_frequency(X, 0.02, 1)
    assert e.value.status == gpu.RG_ERR_INVALID


def test_pipeline_end_to_end(gpu, oracle, tmp_path):
    """Index files -> aligned train/test -> mu, Sigma, realised frequency on
    the GPU -> .bin files -> a resident portfolio that simulates."""
    import importlib.util, os, sys
    here = os.path.dirname(__file__)
    spec = importlib.util.spec_from_file_location("tp", os.path.join(here, "test_preprocess.py"))
    tp = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(tp)
    from riskgpu import preprocess
    files, series = tp.write_index_files(str(tmp_path), seed=21, n_idx=6, days=700)
    cfg = {"start": "2016-01-01", "end": "2017-12-31", "x": 0.02, "k": 2, "train_ratio": 0.8, "indices": files}
    out = preprocess.run_pipeline(cfg, str(tmp_path), str(tmp_path / "data"))
    ref_train, ref_test = oracle.align_and_split(series, dt.date(2016, 1, 1), dt.date(2017, 12, 31), 0.8)
    Xtr = np.array([v for _, v in ref_train], dtype=np.float64)
    Xte = np.array([v for _, v in ref_test], dtype=np.float64)
    mu_ref, sigma_ref = oracle.compute_stats(Xtr)
    assert np.max(np.abs(out["Sigma"] - sigma_ref)) <= 1e-12 * np.max(np.abs(sigma_ref))
    assert out["actual_freq"] == oracle.compute_metrics(Xte, 0.02, 2)
    mu, sigma, freq = preprocess.load_results_binary(str(tmp_path / "data"))
    assert np.array_equal(mu, out["mu"]) and np.array_equal(sigma, out["Sigma"]) and freq == out["actual_freq"]
    port = gpu.Portfolio(mu, sigma)
    r = port.simulate(gpu.make_query(100_000, 67, x=0.02, k=2))
    assert 0.0 <= r["p_crash"] <= 1.0 and r["n_paths"] == 100_000

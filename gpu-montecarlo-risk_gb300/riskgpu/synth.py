"""Seeded synthetic portfolios with the shapes of the benchmark workloads.

The reference estimates its inputs from index CSVs (preprocessing/main.py:8-56,
preprocessing_stats.py:18-21) and stores them as mu.bin / sigma.bin
(save_binary.py:23-45).  No public data set is involved in the benchmark
workloads, so every input here is drawn from numpy's PCG64
(`numpy.random.default_rng(seed)`), always in the order: means, factor
loadings, idiosyncratic vols, weights.

Workloads (sizes are the benchmark's):
  one_factor_20   N=20,  H=1,  M=1e6, equal weights, P(w.R < -2%), 99% VaR/CVaR,
                  crash semantics x=0.02, k=5 (the reference's config.yaml:40-41),
                  data and path seed 42.
  one_factor_50   N=50,  H=1,  M=1e8, Dirichlet(1) weights, threshold -3%,
                  crash semantics x=0.03, k=5, seed 67 (config.yaml:37).
  five_factor_600 N=600, H=10 summed daily draws, M=1e7, Dirichlet(1) weights,
                  portfolio threshold -0.65%, crash semantics x=10%, k=60.
  batch_256       256 portfolios, N~U{10..600}, H~U{1..20}, M log-uniform
                  [1e4, 1e6], 3-factor covariance with a per-portfolio seed,
                  thresholds U(-5%, -1%).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class Portfolio:
    name: str
    mu: np.ndarray          # [N] daily mean returns
    sigma: np.ndarray       # [N, N] daily covariance, row-major
    weights: np.ndarray     # [N]
    horizon: int            # days, draws summed
    n_paths: int
    x: float                # asset crash threshold: R_i < -x
    k: int                  # crash count threshold: S >= k
    port_threshold: float   # portfolio breach: w.R < port_threshold
    var_level: float
    seed: int               # path seed

    @property
    def n(self) -> int:
        return int(self.mu.shape[0])


def one_factor_sigma(rng: np.random.Generator, n: int, market_vol: float = 0.012,
                     beta_range=(0.5, 1.5), idio_range=(0.008, 0.02)):
    """mu_i ~ N(3e-4, (2e-4)^2); Sigma = vol^2 beta beta^T + diag(idio^2)."""
    mu = rng.normal(3e-4, 2e-4, n)
    beta = rng.uniform(beta_range[0], beta_range[1], n)
    idio = rng.uniform(idio_range[0], idio_range[1], n)
    sigma = market_vol ** 2 * np.outer(beta, beta) + np.diag(idio ** 2)
    return mu, sigma, beta, idio


def factor_sigma(rng: np.random.Generator, n: int, n_factors: int, loading_scale: float,
                 idio_range=(0.005, 0.025)):
    """mu_i ~ N(3e-4, (2e-4)^2); B ~ N(0, 1) * loading_scale (N x F);
    Sigma = B B^T + diag(idio^2)."""
    mu = rng.normal(3e-4, 2e-4, n)
    B = rng.normal(0.0, 1.0, (n, n_factors)) * loading_scale
    idio = rng.uniform(idio_range[0], idio_range[1], n)
    sigma = B @ B.T + np.diag(idio ** 2)
    return mu, sigma, B, idio


def one_factor_20(n_paths: int = 1_000_000) -> Portfolio:
    rng = np.random.default_rng(42)
    n = 20
    mu, sigma, _, _ = one_factor_sigma(rng, n)
    w = np.full(n, 1.0 / n)
    return Portfolio("one_factor_20", mu, sigma, w, 1, n_paths, 0.02, 5, -0.02, 0.99, 42)


def one_factor_50(n_paths: int = 100_000_000) -> Portfolio:
    rng = np.random.default_rng(67)
    n = 50
    mu, sigma, _, _ = one_factor_sigma(rng, n)
    w = rng.dirichlet(np.ones(n))
    return Portfolio("one_factor_50", mu, sigma, w, 1, n_paths, 0.03, 5, -0.03, 0.99, 67)


def five_factor_600(n_paths: int = 10_000_000) -> Portfolio:
    rng = np.random.default_rng(600)
    n = 600
    mu, sigma, _, _ = factor_sigma(rng, n, 5, 0.5 * 0.01)
    w = rng.dirichlet(np.ones(n))
    # 10-day horizon: per-asset crash at -10%, 60 of 600 assets (P ~ 1%);
    # portfolio breach below -0.65% (P ~ 1%, about the 99% VaR)
    return Portfolio("five_factor_600", mu, sigma, w, 10, n_paths, 0.10, 60, -0.0065, 0.99, 600)


def batch_256(count: int = 256, base_seed: int = 4096, n_max: int = 600,
              m_range=(1e4, 1e6)) -> list[Portfolio]:
    rng = np.random.default_rng(base_seed)
    out = []
    for b in range(count):
        n = int(rng.integers(10, n_max + 1))
        h = int(rng.integers(1, 21))
        m = int(round(math.exp(rng.uniform(math.log(m_range[0]), math.log(m_range[1])))))
        thr = float(rng.uniform(-0.05, -0.01))
        seed = int(rng.integers(1, 2 ** 31))
        prng = np.random.default_rng(seed)
        mu, sigma, _, _ = factor_sigma(prng, n, 3, 0.5 * 0.01)
        w = prng.dirichlet(np.ones(n))
        out.append(Portfolio(f"batch_{b}", mu, sigma, w, h, m, 0.02 * math.sqrt(h),
                             max(1, n // 10), thr, 0.99, seed))
    return out


def write_reference_bins(p: Portfolio, directory: str, actual_freq: float = 0.0) -> None:
    """Write mu.bin / sigma.bin / params.bin in the reference's format
    (save_binary.py:23-45, read by load_binary.c:5-124): int32 N + N f64;
    int32 rows, int32 cols + row-major f64; one f64."""
    import os
    os.makedirs(directory, exist_ok=True)
    n = p.n
    with open(os.path.join(directory, "mu.bin"), "wb") as f:
        f.write(np.int32(n).tobytes())
        f.write(np.ascontiguousarray(p.mu, dtype=np.float64).tobytes())
    with open(os.path.join(directory, "sigma.bin"), "wb") as f:
        f.write(np.int32(n).tobytes())
        f.write(np.int32(n).tobytes())
        f.write(np.ascontiguousarray(p.sigma, dtype=np.float64).tobytes())
    with open(os.path.join(directory, "params.bin"), "wb") as f:
        f.write(np.float64(actual_freq).tobytes())

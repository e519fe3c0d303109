"""Generate tests/golden/oracle_figures.json: the FP64 oracle's answers for
the benchmark workloads, against which the engine's estimates are stated in
units of their Monte Carlo standard error.

For each workload (riskgpu.synth: one_factor_50, five_factor_600):
  inputs_sha256      sha256 of the float64 bytes of mu, Sigma and the weights,
                     so a reader can check that its synthetic inputs are the
                     ones these figures belong to;
  closed forms       the H-day portfolio return is exactly N(H w.mu, H w'Sigma w):
                     P(w.R < threshold), VaR and CVaR of the loss at `alpha`,
                     and the density of the return at the VaR quantile
                     (oracle/mc_oracle.py: portfolio_closed_form);
  p_crash            P(S >= k), S = #{i : R_i < -x}, in FP64:
                     one factor  - Gauss-Hermite quadrature over the market
                                   factor of a Poisson-binomial tail
                                   (mc_oracle.one_factor_crash_prob);
                     five factors - the factor-conditional Poisson-binomial
                                   tail averaged by randomised quasi-Monte
                                   Carlo (mc_oracle.factor_crash_prob), with
                                   the standard error of its scrambles.

Run from the repository root:  python tests/golden/make_oracle_figures.py
(about ten minutes on 8 cores; the oracle library is built first).
"""
import hashlib
import json
import math
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [os.path.join(ROOT, "gpu-montecarlo-risk_gb300"), os.path.join(ROOT, "oracle")]

import numpy as np  # noqa: E402

import mc_oracle  # noqa: E402
from riskgpu import synth  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "oracle_figures.json")
ALPHA = 0.99


def inputs_sha256(p):
    h = hashlib.sha256()
    for a in (p.mu, p.sigma, p.weights):
        h.update(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    return h.hexdigest()


def closed(p):
    cf = mc_oracle.portfolio_closed_form(p.mu, p.sigma, p.weights, p.horizon, p.port_threshold, ALPHA)
    # density of w.R at its (1 - alpha) quantile, for the standard error of
    # the sample quantile
    z = (-cf["var"] - cf["mean"]) / cf["sd"]
    cf["density_at_var"] = math.exp(-0.5 * z * z) / (math.sqrt(2.0 * math.pi) * cf["sd"])
    # E[(L - VaR)^+ ^2] of the loss L = -w.R, for the standard error of CVaR
    # (Var((L - q)^+) / (1 - alpha)^2 / M): with L ~ N(m_L, s^2),
    # a = (q - m_L)/s, E[(L-q)^+] = s(phi(a) - a Q(a)),
    # E[((L-q)^+)^2] = s^2((1 + a^2) Q(a) - a phi(a))
    mL, s, q = -cf["mean"], cf["sd"], cf["var"]
    a = (q - mL) / s
    phi = math.exp(-0.5 * a * a) / math.sqrt(2.0 * math.pi)
    Q = 0.5 * math.erfc(a / math.sqrt(2.0))
    m1 = s * (phi - a * Q)
    m2 = s * s * ((1.0 + a * a) * Q - a * phi)
    cf["excess_var"] = m2 - m1 * m1
    return cf


def main():
    mc_oracle.build()
    figs = {"alpha": ALPHA}

    t0 = time.time()
    p = synth.one_factor_50(n_paths=1)
    rng = np.random.default_rng(67)
    mu, sigma, beta, idio = synth.one_factor_sigma(rng, p.n)
    assert np.array_equal(sigma, p.sigma)
    pc = mc_oracle.one_factor_crash_prob(mu, beta, 0.012, idio, p.x, p.k, p.horizon, nodes=96)
    figs["one_factor_50"] = dict(inputs_sha256=inputs_sha256(p), n=p.n, horizon=p.horizon, x=p.x, k=p.k,
                                 port_threshold=p.port_threshold, p_crash=pc, p_crash_se=0.0,
                                 p_crash_method="Gauss-Hermite quadrature (96 nodes) over the market factor "
                                                "of the Poisson-binomial tail", **closed(p))
    print(f"one_factor_50: p_crash {pc:.10g} ({time.time() - t0:.1f} s)", flush=True)

    t0 = time.time()
    p = synth.five_factor_600(n_paths=1)
    rng = np.random.default_rng(600)
    mu, sigma, B, idio = synth.factor_sigma(rng, p.n, 5, 0.5 * 0.01)
    assert np.array_equal(sigma, p.sigma)
    log2_points, scrambles = 22, 16
    pc, se = mc_oracle.factor_crash_prob(mu, B, idio, p.x, p.k, p.horizon, log2_points=log2_points,
                                         scrambles=scrambles)
    figs["five_factor_600"] = dict(inputs_sha256=inputs_sha256(p), n=p.n, horizon=p.horizon, x=p.x, k=p.k,
                                   port_threshold=p.port_threshold, p_crash=pc, p_crash_se=se,
                                   p_crash_method=f"factor-conditional Poisson-binomial tail, randomised QMC: "
                                                  f"{scrambles} scrambled Sobol' sets of 2^{log2_points} points",
                                   **closed(p))
    print(f"five_factor_600: p_crash {pc:.10g} +- {se:.3g} ({time.time() - t0:.1f} s)", flush=True)

    with open(OUT, "w") as f:
        json.dump(figs, f, indent=1, sort_keys=True)
        f.write("\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()

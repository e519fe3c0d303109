"""Parity at the benchmark workloads' full sizes, through size-independent
properties (per-path checks against the oracle run at small sizes elsewhere):

  * path-range additivity: the draws are keyed by (seed, path index), so the
    counts over [0, M) equal the sum of the counts over [0, c) and [c, M) for
    a cut c that is not a multiple of any tile width;
  * determinism: a repeated launch gives identical 64-bit counts;
  * agreement with the FP64 oracle within 3 Monte Carlo standard errors
    (tests/golden/oracle_figures.json: Gauss-Hermite P(S >= k) for the
    one-factor workload, the factor-conditional oracle for the five-factor
    one, the Gaussian closed form for P(breach); the oracle's own error is
    added in quadrature).

Workloads: one_factor_50 (N = 50, 1e8 paths, the drop-in) on the plain FP32
kernel; five_factor_600 (N = 600, H = 10 summed daily draws, 1e7 paths) on
the BF16x3 tensor-core form and the plain FP32 kernel.
"""
import json
import math
import os

import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _counts(gpu, port, p, M, prec, offset=0):
    import torch
    d = torch.zeros(2, dtype=torch.int64, device="cuda")
    q = gpu.make_query(M, p.seed, x=p.x, k=p.k, horizon=p.horizon, port_threshold=p.port_threshold,
                       precision=prec, path_offset=offset)
    port.launch_counts(q, d.data_ptr())
    torch.cuda.synchronize()
    return tuple(int(v) for v in d.cpu().tolist())


def _fig(name):
    return json.load(open(os.path.join(GOLDEN, "oracle_figures.json")))[name]


def _within_3se(count, M, p_ref, se_ref=0.0):
    p = count / M
    se = math.sqrt(p_ref * (1 - p_ref) / M + se_ref * se_ref)
    return abs(p - p_ref) < 3 * se, (p, p_ref, (p - p_ref) / se)


@pytest.mark.parametrize("workload,prec_name", [("one_factor_50", "fp32"), ("five_factor_600", "bf16x3"),
                                                ("five_factor_600", "fp32")])
def test_full_size_additivity_determinism_and_oracle(gpu, workload, prec_name):
    from riskgpu import synth
    M = 100_000_000 if workload == "one_factor_50" else 10_000_000
    p = getattr(synth, workload)(n_paths=M)
    prec = {"fp32": gpu.PREC_FP32, "bf16x3": gpu.PREC_BF16X3}[prec_name]
    port = gpu.Portfolio(p.mu, p.sigma, p.weights)
    whole = _counts(gpu, port, p, M, prec)
    assert _counts(gpu, port, p, M, prec) == whole  # deterministic
    cut = M // 3 + 12_345  # not a multiple of 32, 64 or 96 paths
    a = _counts(gpu, port, p, cut, prec)
    b = _counts(gpu, port, p, M - cut, prec, offset=cut)
    assert (a[0] + b[0], a[1] + b[1]) == whole
    fig = _fig(workload)
    assert fig["inputs_sha256"] and fig["k"] == p.k and fig["port_threshold"] == p.port_threshold
    ok, info = _within_3se(whole[0], M, fig["p_crash"], fig["p_crash_se"])
    assert ok, ("P(S >= k)", info)
    ok, info = _within_3se(whole[1], M, fig["p_breach"])
    assert ok, ("P(breach)", info)
    port.close()

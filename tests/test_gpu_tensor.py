"""The tcgen05 precision form against the oracle, per path, through the C ABI.

Tolerances of the tensor-core form (FP32 accumulation of split products):
  FP16x3 (FP16 hi+lo of Z and of 2^8 L, three products): asset returns
    within NEAR_FP16 = 1e-5 of the FP64 value decide S identically; w.R
    within 5e-5;
  BF16x3: NEAR_BF16 = 4e-5; w.R within 2e-4.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {"fp16x3": (3, 1e-5, 5e-5), "bf16x3": (1, 4e-5, 2e-4)}


def _run(gpu, port, M, seed, x, k, thr, horizon, prec, draw_mode=0, var_level=0.0):
    import torch
    S = torch.full((M,), -1, dtype=torch.int32, device="cuda")
    W = torch.full((M,), float("nan"), dtype=torch.float32, device="cuda")
    q = gpu.make_query(M, seed, x=x, k=k, horizon=horizon, port_threshold=thr, precision=prec,
                       d_s_values=S.data_ptr(), d_port_values=W.data_ptr(), draw_mode=draw_mode,
                       var_level=var_level)
    r = port.simulate(q)
    torch.cuda.synchronize()
    return r, S.cpu().numpy(), W.cpu().numpy().astype(np.float64)


def _case(n, seed):
    from riskgpu import synth
    rng = np.random.default_rng(seed)
    mu, sigma, _, _ = synth.factor_sigma(rng, n, 5, 0.5 * 0.01)
    w = rng.dirichlet(np.ones(n))
    return mu, sigma, w


@pytest.mark.parametrize("prec", ["fp16x3", "bf16x3"])
@pytest.mark.parametrize("n,horizon,M", [(16, 1, 256), (64, 1, 1000), (130, 2, 777), (600, 10, 256)])
def test_tc_per_path_parity(gpu, oracle, prec, n, horizon, M):
    code, near_tol, port_tol = CASES[prec]
    mu, sigma, w = _case(n, n + 1)
    x, k, thr, seed = 0.02 * math.sqrt(horizon), max(1, n // 10), -0.03, 5 + n
    port = gpu.Portfolio(mu, sigma, w)
    r, S, W = _run(gpu, port, M, seed, x, k, thr, horizon, code)
    L_ref, _ = oracle.cholesky_lower(sigma)
    ref = oracle.mc_philox(mu, L_ref, w, horizon, M, seed, x, k, thr, want_S=True, want_port=True, want_R=True)
    assert np.isfinite(W).all()
    assert np.max(np.abs(W - ref["port"])) <= port_tol, np.max(np.abs(W - ref["port"]))
    near = np.min(np.abs(ref["R"] + x), axis=1) < near_tol
    bad = (S != ref["S"]) & ~near
    assert not bad.any(), f"{int(bad.sum())} paths differ; first {np.nonzero(bad)[0][:5]}"
    assert r["crash_count"] == int((S >= k).sum())
    assert r["breach_count"] == int((W < thr).sum())

"""The allocation-free entry point, rg_simulate_noalloc, through the C ABI.

For callers that cannot call cudaMalloc where they run a query (a host that
budgets every device byte itself, a latency-critical loop, a plugin whose
framework owns the device heap).  It must give what rg_simulate gives for
the same portfolio and query: exact 64-bit counts, the same VaR order
statistic, CVaR within 1e-9 relative (the two sum the tail in different
orders), on two calls in a row (the second call finds the previous call's
data in the shared scratch array and must clear what it relies on).

The tensor-core forms (FP16x3, BF16x3) go through the same entry point and
report a bounded wait that ran out as RG_ERR_TIMEOUT, like rg_simulate.

Collected last (file name) so that a failure here comes after every other
test has run; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(engine, port, q):
    r = engine.Result()
    st = engine.lib().rg_simulate_noalloc(port.handle, ctypes.byref(q), ctypes.byref(r), None)
    return st, r.as_dict()


def _same(a, b):
    assert a["crash_count"] == b["crash_count"]
    assert a["breach_count"] == b["breach_count"]
    assert a["p_crash"] == b["p_crash"] and a["se_crash"] == b["se_crash"]
    if np.isnan(b["var"]):
        assert np.isnan(a["var"]) and np.isnan(a["cvar"])
    else:
        assert a["tail_count"] == b["tail_count"]
        assert a["var"] == b["var"]
        assert abs(a["cvar"] - b["cvar"]) <= 1e-9 * abs(b["cvar"])
        assert a["var_passes"] == b["var_passes"]


@pytest.mark.parametrize("var_level", [0.99, 0.0])
def test_noalloc_matches_rg_simulate_twice(gpu, var_level):
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=1)
    port = gpu.Portfolio(p.mu, p.sigma, p.weights)
    queries = [gpu.make_query(4_000_000, 67, x=p.x, k=p.k, port_threshold=p.port_threshold,
                              var_level=var_level),
               gpu.make_query(1_500_001, 68, x=p.x, k=p.k, port_threshold=p.port_threshold,
                              var_level=var_level, horizon=2)]
    for q in queries:  # two calls in a row, different queries
        ref = port.simulate(q)
        st, got = _noalloc(gpu, port, q)
        assert st == gpu.RG_OK, gpu.lib().rg_last_error()
        _same(got, ref)


def test_noalloc_histogram_fallback(gpu, monkeypatch):
    """The displaced-band injection forces both entry points through the
    histogram and bin-select passes; results still agree."""
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=1)
    port = gpu.Portfolio(p.mu, p.sigma, p.weights)
    monkeypatch.setenv("RG_FAULT_INJECT", "varband")
    q = gpu.make_query(2_000_000, 5, x=p.x, k=p.k, port_threshold=p.port_threshold, var_level=0.99)
    ref = port.simulate(q)
    assert ref["var_passes"] == 3
    for _ in range(2):
        st, got = _noalloc(gpu, port, q)
        assert st == gpu.RG_OK, gpu.lib().rg_last_error()
        _same(got, ref)


def test_noalloc_rejects_oversized_queries(gpu):
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=1)
    port = gpu.Portfolio(p.mu, p.sigma, p.weights)
    q = gpu.make_query(2_000_000_000, 1, var_level=0.99)
    st, _ = _noalloc(gpu, port, q)
    assert st == gpu.RG_ERR_UNSUPPORTED
    assert b"scratch array" in gpu.lib().rg_last_error()


def _factor_case(gpu, n, seed):
    from riskgpu import synth
    rng = np.random.default_rng(seed)
    mu, sigma, _, _ = synth.factor_sigma(rng, n, 5, 0.5 * 0.01)
    w = rng.dirichlet(np.ones(n))
    return gpu.Portfolio(mu, sigma, w)


@pytest.mark.parametrize("var_level", [0.99, 0.0])
@pytest.mark.parametrize("prec", ["fp16x3", "bf16x3"])
def test_noalloc_tensor_forms_match_rg_simulate(gpu, prec, var_level):
    """The tcgen05 kernels through the allocation-free entry point give the
    same counts and VaR order statistic as through rg_simulate, on two
    calls in a row."""
    code = {"fp16x3": gpu.PREC_FP16X3, "bf16x3": gpu.PREC_BF16X3}[prec]
    port = _factor_case(gpu, 300, 29)
    queries = [gpu.make_query(300_000, 3, x=0.05, k=30, horizon=5, port_threshold=-0.04,
                              precision=code, var_level=var_level),
               gpu.make_query(120_001, 4, x=0.03, k=20, horizon=2, port_threshold=-0.03,
                              precision=code, var_level=var_level)]
    for q in queries:
        ref = port.simulate(q)
        st, got = _noalloc(gpu, port, q)
        assert st == gpu.RG_OK, gpu.lib().rg_last_error()
        _same(got, ref)


@pytest.mark.parametrize("var_level", [0.99, 0.0])
def test_noalloc_tensor_bounded_wait_reports_timeout(gpu, monkeypatch, var_level):
    """Failure detection without a GPU fault: RG_FAULT_INJECT=tcstall leaves
    one pipeline stage of the tensor-core kernel unfilled, its bounded wait
    runs out and it sets its error word; the allocation-free entry point
    returns RG_ERR_TIMEOUT instead of incomplete counts, and the next call
    on the same context succeeds."""
    port = _factor_case(gpu, 200, 3)
    q = gpu.make_query(65_536, 1, x=0.02, k=5, port_threshold=-0.03, precision=gpu.PREC_BF16X3,
                       var_level=var_level)
    monkeypatch.setenv("RG_FAULT_INJECT", "tcstall")
    st, _ = _noalloc(gpu, port, q)
    assert st == gpu.RG_ERR_TIMEOUT, gpu.lib().rg_last_error()
    assert b"bounded wait" in gpu.lib().rg_last_error()
    monkeypatch.delenv("RG_FAULT_INJECT")
    st, got = _noalloc(gpu, port, q)
    assert st == gpu.RG_OK, gpu.lib().rg_last_error()
    _same(got, port.simulate(q))

"""The tcgen05 precision form against the oracle, per path, through the C ABI.

Tolerances of the tensor-core form (FP32 accumulation of split products):
  FP16x3 (FP16 hi+lo of Z and of 2^8 L, three products): asset returns
    within NEAR_FP16 = 1e-5 of the FP64 value decide S identically; w.R
    within 5e-5;
  BF16x3: NEAR_BF16 = 4e-5; w.R within 2e-4.
"""
import math
import os

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


# the tcgen05 kernels: "ws" (warp-specialised, the default: 128-path tiles up
# to four row tiles, N <= 511; 96 up to five, N <= 639; else 64; the Lhat
# copies issued by their own warp with aggregated draws, by the MMA thread
# with daily draws), "ws-split" / "ws-merged" (either copy issuer forced),
# "ws96" and "ws64" (its tile capped at 96 / 64 paths) and "simple"
# (phase-serial, 64-path tiles); RG_TC_KERNEL forces one of them
KERNELS = ["ws", "ws-split", "ws-merged", "ws96", "ws64", "simple"]


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("prec", ["fp16x3", "bf16x3"])
@pytest.mark.parametrize("n,horizon,M", [(1, 1, 300), (16, 1, 256), (64, 1, 1000), (130, 2, 777), (511, 1, 300),
                                         (512, 1, 300), (600, 10, 256), (639, 1, 200), (640, 2, 200)])
def test_tc_per_path_parity(gpu, oracle, monkeypatch, kernel, prec, n, horizon, M):
    monkeypatch.setenv("RG_TC_KERNEL", kernel)
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


@pytest.mark.parametrize("M,offset", [(1, 0), (5, 3), (95, 0), (97, 1), (193, 1_000_003)])
def test_tc_ragged_path_counts(gpu, oracle, M, offset):
    """Tiles the paths fill only in part (1 path, one short of or one past a
    96-path tile, an offset far from 0): every written path equals the oracle
    and no slot past M is touched."""
    import torch
    n, horizon = 130, 2
    code, near_tol, port_tol = CASES["bf16x3"]
    mu, sigma, w = _case(n, 7)
    x, k, thr, seed = 0.02 * math.sqrt(horizon), 13, -0.03, 91
    port = gpu.Portfolio(mu, sigma, w)
    S = torch.full((M + 8,), -1, dtype=torch.int32, device="cuda")
    W = torch.full((M + 8,), float("nan"), dtype=torch.float32, device="cuda")
    q = gpu.make_query(M, seed, x=x, k=k, horizon=horizon, port_threshold=thr, precision=code,
                       d_s_values=S.data_ptr(), d_port_values=W.data_ptr(), path_offset=offset)
    r = port.simulate(q)
    torch.cuda.synchronize()
    S, W = S.cpu().numpy(), W.cpu().numpy().astype(np.float64)
    assert (S[M:] == -1).all() and np.isnan(W[M:]).all()
    S, W = S[:M], W[:M]
    L_ref, _ = oracle.cholesky_lower(sigma)
    ref = oracle.mc_philox(mu, L_ref, w, horizon, M, seed, x, k, thr, want_S=True, want_port=True, want_R=True,
                           path_offset=offset)
    assert np.max(np.abs(W - ref["port"])) <= port_tol
    near = np.min(np.abs(ref["R"] + x), axis=1) < near_tol
    assert not ((S != ref["S"]) & ~near).any()
    assert r["crash_count"] == int((S >= k).sum()) and r["breach_count"] == int((W < thr).sum())
    port.close()


@pytest.mark.parametrize("kernel", KERNELS)
def test_tc_path_ranges_add_up(gpu, monkeypatch, kernel):
    """Counter-based draws: counts over [0, M) equal the sum over a split at
    an offset that is not a multiple of the 64-path tile."""
    monkeypatch.setenv("RG_TC_KERNEL", kernel)
    mu, sigma, w = _case(300, 17)
    port = gpu.Portfolio(mu, sigma, w)
    M, cut = 50_000, 20_011
    def run(n, off):
        q = gpu.make_query(n, 41, x=0.03, k=20, horizon=3, port_threshold=-0.03, precision=3)
        q.path_offset = off
        return port.simulate(q)
    whole, a, b = run(M, 0), run(cut, 0), run(M - cut, cut)
    assert whole["crash_count"] == a["crash_count"] + b["crash_count"]
    assert whole["breach_count"] == a["breach_count"] + b["breach_count"]


@pytest.mark.parametrize("kernel", KERNELS)
def test_tc_bounded_wait_reports_timeout(gpu, monkeypatch, kernel):
    """Failure detection without a GPU fault: with RG_FAULT_INJECT=tcstall
    one pipeline stage is never filled, the kernel's bounded wait (2 s) runs
    out, it drains its own copies and MMAs, frees its tensor memory and sets
    its error word; the host returns RG_ERR_TIMEOUT and the context stays
    usable for the next query."""
    mu, sigma, w = _case(200, 3)
    port = gpu.Portfolio(mu, sigma, w)
    q = gpu.make_query(4096, 1, x=0.02, k=5, precision=3)
    monkeypatch.setenv("RG_TC_KERNEL", kernel)
    monkeypatch.setenv("RG_FAULT_INJECT", "tcstall")
    with pytest.raises(gpu.RiskGpuError) as e:
        port.simulate(q)
    assert e.value.status == gpu.RG_ERR_TIMEOUT
    monkeypatch.delenv("RG_FAULT_INJECT")
    r = port.simulate(q)
    assert r["n_paths"] == 4096


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("prec", ["fp16x3", "bf16x3"])
def test_tc_var_and_aggregated(gpu, oracle, monkeypatch, kernel, prec):
    """VaR/CVaR order statistics of the tensor-core form equal those of its
    own per-path returns; aggregated draws match the oracle per path."""
    monkeypatch.setenv("RG_TC_KERNEL", kernel)
    code, near_tol, port_tol = CASES[prec]
    mu, sigma, w = _case(300, 11)
    port = gpu.Portfolio(mu, sigma, w)
    r, S, W = _run(gpu, port, 200_000, 3, 0.05, 30, -0.04, 5, code, var_level=0.99)
    var, cvar, T = oracle.var_cvar(W, 0.99)
    assert r["tail_count"] == T and r["var"] == var and abs(r["cvar"] - cvar) <= 1e-9 * abs(cvar)
    M = 2000
    r, S, W = _run(gpu, port, M, 9, 0.05, 30, -0.04, 5, code, draw_mode=1)
    L_ref, _ = oracle.cholesky_lower(sigma)
    ref = oracle.mc_philox(mu, L_ref, w, 5, M, 9, 0.05, 30, -0.04, want_S=True, want_port=True, want_R=True,
                           aggregated=True)
    assert np.max(np.abs(W - ref["port"])) <= port_tol
    near = np.min(np.abs(ref["R"] + 0.05), axis=1) < near_tol
    assert not ((S != ref["S"]) & ~near).any()


def test_tc_statistics_vs_fp32_and_closed_form(gpu, oracle):
    """All forms agree at equal tail-probability error: at N = 600, H = 10
    (the precision-form workload) each form's estimates lie within 3 Monte
    Carlo standard errors of the FP64 oracle -- P(w.R < threshold), VaR and
    CVaR against their Gaussian closed forms, P(S >= k) against the
    factor-conditional Poisson-binomial oracle (tests/golden/
    oracle_figures.json, whose own error is added in quadrature)."""
    import json
    from conftest import GOLDEN
    from riskgpu import synth
    p = synth.five_factor_600(n_paths=1)
    fig = json.load(open(os.path.join(GOLDEN, "oracle_figures.json")))["five_factor_600"]
    assert fig["port_threshold"] == p.port_threshold and fig["k"] == p.k and fig["x"] == p.x
    port = gpu.Portfolio(p.mu, p.sigma, p.weights)
    M, alpha = 4_000_000, 0.99
    cf = oracle.portfolio_closed_form(p.mu, p.sigma, p.weights, p.horizon, p.port_threshold, alpha)
    se_b = math.sqrt(cf["p_breach"] * (1 - cf["p_breach"]) / M)
    se_c = math.sqrt(fig["p_crash"] * (1 - fig["p_crash"]) / M + fig["p_crash_se"] ** 2)
    se_q = math.sqrt(alpha * (1 - alpha) / M) / fig["density_at_var"]
    se_cv = math.sqrt(fig["excess_var"] / M) / (1 - alpha)
    for prec in (gpu.PREC_FP32, gpu.PREC_BF16X3, gpu.PREC_FP16X3):
        r = port.simulate(gpu.make_query(M, 21, x=p.x, k=p.k, horizon=p.horizon, port_threshold=p.port_threshold,
                                         precision=prec, var_level=alpha))
        assert abs(r["p_breach"] - cf["p_breach"]) < 3 * se_b, (prec, r["p_breach"], cf["p_breach"])
        assert abs(r["p_crash"] - fig["p_crash"]) < 3 * se_c, (prec, r["p_crash"], fig["p_crash"])
        assert abs(r["var"] - cf["var"]) < 3 * se_q, (prec, r["var"], cf["var"])
        assert abs(r["cvar"] - cf["cvar"]) < 3 * se_cv, (prec, r["cvar"], cf["cvar"])


# ------------------------------------------------------------------ batches
def _batch_items(gpu, count, seed=4096, m_range=(2e3, 6e4), n_max=600):
    from riskgpu import synth
    ps = synth.batch_256(count=count, base_seed=seed, n_max=n_max, m_range=m_range)
    items = []
    for p in ps:
        port = gpu.Portfolio(p.mu, p.sigma, p.weights)
        q = gpu.make_query(p.n_paths, p.seed, x=p.x, k=p.k, horizon=p.horizon,
                           port_threshold=p.port_threshold, precision=3)
        items.append((port, q))
    return ps, items


@pytest.mark.parametrize("flags", [0, 1])
def test_batch_equals_individual_queries(gpu, flags):
    """Each item's counts from one persistent batched launch equal the counts
    of the same query run alone (same per-path arithmetic, integer counts):
    results do not depend on batching.  With and without the CUDA graph;
    two launches of the same batch agree."""
    ps, items = _batch_items(gpu, 24)
    batch = gpu.Batch(items, flags=flags)
    res = batch.run()
    res2 = batch.run()
    for (port, q), r, r2 in zip(items, res, res2):
        alone = port.simulate(q)
        assert (r["crash_count"], r["breach_count"]) == (alone["crash_count"], alone["breach_count"])
        assert (r2["crash_count"], r2["breach_count"]) == (r["crash_count"], r["breach_count"])
    inf = batch.info()
    assert inf["graph"] == (0 if flags else 1) and inf["items"] == 24


def test_batch_mixed_precisions_and_draw_modes(gpu):
    """One persistent launch over items that differ in precision (FP16x3 and
    BF16x3), draw mode (daily, aggregated), horizon, asset count and path
    budget: each item's counts equal the same query alone, in either order."""
    from riskgpu import synth
    ps = synth.batch_256(count=12, base_seed=99, n_max=600, m_range=(3e3, 3e4))
    items = []
    for i, p in enumerate(ps):
        port = gpu.Portfolio(p.mu, p.sigma, p.weights)
        q = gpu.make_query(p.n_paths, p.seed, x=p.x, k=p.k, horizon=p.horizon,
                           port_threshold=p.port_threshold, precision=(3 if i % 2 == 0 else 1),
                           draw_mode=(i // 2) % 2)
        items.append((port, q))
    alone = [port.simulate(q) for port, q in items]
    for order in (list(range(12)), list(reversed(range(12)))):
        res = gpu.Batch([items[i] for i in order]).run()
        for i, r in zip(order, res):
            assert (r["crash_count"], r["breach_count"]) == (alone[i]["crash_count"], alone[i]["breach_count"]), i


def test_batch_with_six_row_tiles_uses_64_path_tiles(gpu):
    """An N = 640 item (six row tiles: 6 x 96 columns would not fit in
    tensor memory) moves the whole batch to 64-path tiles; counts still
    equal the queries alone."""
    items = []
    for i, n in enumerate((640, 37, 300)):
        mu, sigma, w = _case(n, 50 + i)
        port = gpu.Portfolio(mu, sigma, w)
        q = gpu.make_query(9_000 + 1_000 * i, 7 + i, x=0.03, k=max(1, n // 12), horizon=2,
                           port_threshold=-0.03, precision=3)
        items.append((port, q))
    res = gpu.Batch(items).run()
    for (port, q), r in zip(items, res):
        alone = port.simulate(q)
        assert (r["crash_count"], r["breach_count"]) == (alone["crash_count"], alone["breach_count"])


def test_server_rejects_six_row_tiles(gpu):
    """The served form runs 96-path tiles: N = 640 is refused at
    registration, N = 639 is accepted."""
    srv = gpu.Server()
    try:
        mu, sigma, w = _case(640, 3)
        with pytest.raises(gpu.RiskGpuError) as e:
            srv.register(1, gpu.Portfolio(mu, sigma, w))
        assert e.value.status == gpu.RG_ERR_UNSUPPORTED
        mu, sigma, w = _case(639, 3)
        port = gpu.Portfolio(mu, sigma, w)
        srv.register(2, port)
    finally:
        srv.close()


def test_batch_autotuner_persists_choice(gpu, tmp_path, monkeypatch):
    monkeypatch.setenv("RG_TUNE_CACHE", str(tmp_path / "tune.json"))
    ps, items = _batch_items(gpu, 12, seed=7)
    b = gpu.Batch(items)
    before = b.run()
    b.tune()
    after = b.run()
    assert [(r["crash_count"], r["breach_count"]) for r in before] == \
           [(r["crash_count"], r["breach_count"]) for r in after]
    inf = b.info()
    assert inf["tuned"] == 1
    import json
    cache = json.load(open(tmp_path / "tune.json"))
    assert len(cache) == 1 and list(cache.values())[0][:2] == [inf["unit_tiles"], inf["ctas_per_sm"]]
    b2 = gpu.Batch(items)
    assert b2.info()["tuned"] == 1 and b2.info()["unit_tiles"] == inf["unit_tiles"]


def test_batch_rejects_unsupported_items(gpu):
    from riskgpu import synth
    p = synth.one_factor_20(n_paths=1)
    port = gpu.Portfolio(p.mu, p.sigma, p.weights)
    with pytest.raises(gpu.RiskGpuError):
        gpu.Batch([(port, gpu.make_query(1000, 1, var_level=0.99, precision=3))])
    with pytest.raises(gpu.RiskGpuError):
        gpu.Batch([(port, gpu.make_query(1000, 1, rng=gpu.RNG_XORWOW_REF))])


# ------------------------------------------------------------------ serving
def test_server_results_equal_alone_and_in_the_mix(gpu):
    """Continuous batching: many requests from several client threads,
    arriving while others run; every result equals the same query run
    alone (integer counts, exactly)."""
    import threading
    ps, items = _batch_items(gpu, 16, seed=99, m_range=(1e3, 2e4))
    srv = gpu.Server(slots=3, max_batch_items=8, poll_us=20)
    for i, (port, _) in enumerate(items):
        srv.register(i, port)
    results = {}

    def client(ids):
        for rep in range(3):
            for i in ids:
                tk = srv.submit(i, items[i][1])
                results[(i, rep, threading.get_ident())] = srv.wait(tk)

    th = [threading.Thread(target=client, args=(list(range(j, 16, 4)),)) for j in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    alone = [port.simulate(q) for port, q in items]
    assert len(results) == 16 * 3
    for (i, rep, _), r in results.items():
        assert (r["crash_count"], r["breach_count"]) == (alone[i]["crash_count"], alone[i]["breach_count"])
        assert r["latency_ms"] > 0
    st = srv.stats()
    assert st["completed"] == 48 and st["p99_ms"] >= st["p50_ms"] > 0
    assert st["batches"] >= 1
    srv.close()


def test_server_admission_by_headroom(gpu):
    """With a headroom larger than the device, requests are never admitted and
    fail with RG_ERR_ADMISSION after the admission timeout; a server with a
    normal headroom serves the same request."""
    ps, items = _batch_items(gpu, 1, seed=5, m_range=(1e3, 2e3))
    port, q = items[0]
    srv = gpu.Server(headroom_bytes=1 << 60, admission_timeout_ms=200.0)
    srv.register(0, port)
    st, _ = srv.try_wait(srv.submit(0, q))
    assert st == gpu.RG_ERR_ADMISSION
    assert srv.stats()["refused"] == 1
    srv.close()
    srv = gpu.Server()
    srv.register(0, port)
    r = srv.wait(srv.submit(0, q))
    assert r["crash_count"] == port.simulate(q)["crash_count"]
    srv.close()

"""Benchmark: paths/s of the tensor-core precision form against the plain FP32
kernel at equal tail-probability error, plus the served p50/p99 latency.

Default workload (the configuration the headline metric is quoted on):
  five_factor_600  N = 600 assets, covariance B B^T + diag(idio^2) from 5
                   factors (loadings N(0, 0.5^2) * 0.01, idiosyncratic vol
                   U(0.005, 0.025)), 10-day horizon with summed daily draws,
                   M = 1e7 paths per step, Dirichlet(1) weights, portfolio
                   threshold -0.65%, crash semantics x = 10%, k = 60, seed 600,
                   Philox normals, FP64 Cholesky on the GPU (resident).
                   Synthetic inputs (numpy PCG64), no data set.
  A step is one pass of one kernel over the M paths (breach and crash
  counts of every path, exact 64-bit integers).

`value`       paths/s of the BF16x3 tensor-core form (Z . L^T on tcgen05 in
              BF16 hi+lo with FP32 accumulation), factor resident in HBM,
              device time of the K timed kernels (CUDA events on the
              launching stream).  The inputs are a few MB, so L2 is flushed
              (a 256 MB write) before every timed step, outside the events.
`plain_fp32`  the plain FP32 kernel (same draws, same counts) timed the same
              way in the same run; `ratio_vs_plain_fp32` = value / it.
`se_units`    each form's estimates against the FP64 oracle's figures for
              these inputs (P(breach), VaR and CVaR in closed form; P(S >= k)
              from the factor-conditional Poisson-binomial oracle), as
              (estimate - oracle) / standard error.  The figures come from
              tests/golden/oracle_figures.json; its input checksum is
              checked.
`e2e`         the same metric through the public C ABI with host buffers
              (rg_run: mu, Sigma and weights uploaded from pinned host
              memory, factored on the GPU, tensor tiles built, kernel run,
              counts read back) every step.
`served`      Poisson arrivals at 2,000 queries/s of 1e5-path queries over
              64 resident portfolios through the server (continuous
              batching): p50/p99 latency and paths/s, against per-query
              launches of the plain kernel.
`batched`     256 portfolios (N ~ U{10..600}, H ~ U{1..20}, M log-uniform
              [1e4, 1e6]) in one persistent tensor-core launch replayed from
              a CUDA graph, against per-portfolio plain FP32 launches.
`one_factor_50` the drop-in workload (N = 50, H = 1, 1e8 paths) on the plain
              fused FP32 kernel, device and through get_cuda_model().
`roofline`    the tensor-core kernel: normals/s against the measured
              normal-generation peak (the bound with daily draws) and useful
              tensor FLOP/s against the measured BF16 peak.
`cpu_baseline` the reference's serial CPU model on the host (1 core), bounded
              sample.

--impl reference times the reference's CPU implementation of this path (its
serial and OpenMP models; compiled from the reference's sources where the
reference tree exists, else the oracle's restatement of them) on all host
cores, on a bounded sample of the same workload.
"""
import argparse
import contextlib
import dataclasses
import hashlib
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "gpu-montecarlo-risk_gb300"))

METRIC = "paths_per_second"
UNIT = "paths/s"
ALPHA = 0.99
ORACLE_FIGURES = os.path.join(ROOT, "tests", "golden", "oracle_figures.json")

# DRAM bytes (read + write) per launch from ncu captures; neither grows with
# the paths per launch (no per-path data leaves the chip).
#   mc_rows_kernel at N = 50: 41.2 KB read + 1.3 KB written (the factor in
#   parameter space, the counters)
#   mc_tcws_kernel at N = 600: the Lhat tiles read once, about 1.0 MB
NCU_TRAFFIC_BYTES = {"one_factor_50": 42_496, "five_factor_600": 1_000_000}

# Thread instructions the tcgen05 kernel issues per normal it draws, daily
# draws at N = 600, H = 10 (ncu smsp__inst_executed.sum of a 1e6-path launch,
# 3.527e9 warp instructions x 32 / 6e9 normals).  With the SM count and the
# sampled SM clock it gives the kernel's issue bound: every SM issuing 4 warp
# instructions (128 thread instructions) a cycle.
TC_THREAD_INST_PER_NORMAL = 18.8
# The same for the fused N = 50 kernel (mc_rows_kernel<13, true, false>):
# thread instructions a path (ncu, 6.73e8 warp instructions for 1e7 paths;
# 52 normals at about 15.8 instructions each plus 663 FFMA2, their L loads
# and the per-row work).
ROWS_THREAD_INST_PER_PATH = 2155


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="riskgpu", choices=["riskgpu", "reference"])
    ap.add_argument("--paths", type=int, default=None,
                    help="paths per step (default: the workload's, 1e7 or 1e8)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="approximate CPU time of the bounded CPU samples")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline forms only (no served, batched or one_factor_50 sub-records)")
    ap.add_argument("--workload", default="five_factor_600",
                    choices=["five_factor_600", "one_factor_50", "batch_256", "served"],
                    help="five_factor_600 (N=600, H=10, 1e7 paths per step) is the headline; "
                         "one_factor_50 is the drop-in workload alone")
    ap.add_argument("--horizon", type=int, default=None,
                    help="override five_factor_600's 10-day horizon (instruction-count sweeps over the "
                         "horizon; the headline uses the workload's own)")
    ap.add_argument("--draw-mode", default="daily", choices=["daily", "aggregated"])
    ap.add_argument("--precision", default="auto", choices=["auto", "fp32", "bf16x3", "fp16x3"],
                    help="auto: bf16x3 for five_factor_600, fp32 for one_factor_50")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(args):
    """The synthetic portfolio of the workload, sized to the paths per step."""
    from riskgpu import synth
    if args.horizon is not None and args.workload != "five_factor_600":
        raise SystemExit("--horizon applies to the five_factor_600 workload only")
    if args.workload == "one_factor_50":
        if args.paths is None:
            args.paths = 100_000_000
        return synth.one_factor_50(n_paths=args.paths)
    if args.paths is None:
        args.paths = 10_000_000
    p = synth.five_factor_600(n_paths=args.paths)
    if args.horizon is not None:
        if args.horizon < 1:
            raise SystemExit("--horizon must be >= 1")
        p = dataclasses.replace(p, horizon=args.horizon)
    return p


def precision_name(args):
    if args.precision != "auto":
        return args.precision
    return "fp32" if args.workload == "one_factor_50" else "bf16x3"


def config(args, world, p):
    return {"workload": args.workload, "n_assets": p.n, "horizon_days": p.horizon,
            "paths_per_step": args.paths,
            "factor": "one-factor" if p.n == 50 else "five-factor", "weights": "Dirichlet(1)",
            "port_threshold": p.port_threshold, "x": p.x, "k": p.k, "rng": "philox4x32-10",
            "draws": args.draw_mode + (" (H normals per asset, summed)" if args.draw_mode == "daily" else
                                       " (one N(0, H) draw per asset)"),
            "precision": precision_name(args),
            "cholesky": "fp64 on GPU, resident", "l2": "flushed (256 MB write) before each timed step",
            "parallelism": f"path-range shards x{world}" if world > 1 else "1 GPU"}


def measured_peaks():
    """The measured HBM / BF16 peaks of this machine, else the fallback."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return {"bf16_tflops": float(d["bf16_tflops"]), "hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    except (OSError, KeyError, ValueError):
        return {"bf16_tflops": 1900.0, "hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


@contextlib.contextmanager
def quiet_stdout():
    """Silence stdout at the file-descriptor level: the reference's models
    print with C stdio, which Python's redirect does not catch."""
    import ctypes
    libc = ctypes.CDLL(None)
    sys.stdout.flush()
    libc.fflush(None)
    saved = os.dup(1)
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    try:
        yield
    finally:
        libc.fflush(None)
        os.dup2(saved, 1)
        os.close(saved)
        os.close(devnull)


# ------------------------------------------------------------------ CPU legs
def cpu_sample_paths(rate_guess, seconds):
    return max(200, int(rate_guess * seconds))


def run_cpu_reference(p, seconds, threads):
    """The reference's CPU models on a bounded sample: (kind, details).  The
    reference's models have no horizon or weights: each path is one day of
    N normals and a full N x N dgemv (its per-path work at H = 10 would only
    add normals, so this rate bounds the H-day rate from above)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import mc_oracle
    mc_oracle.build()
    use_ref = mc_oracle.ref_available()
    kind = "reference" if use_ref else "port"
    out = {}
    for model, nthreads in (("serial", 1), ("openmp", threads)):
        # calibrate on a small sample, then run ~seconds of work
        M0 = 2000 if p.n <= 64 else 200
        t0 = time.perf_counter()
        _cpu_run(mc_oracle, use_ref, model, p, M0, nthreads)
        rate0 = M0 / max(time.perf_counter() - t0, 1e-6)
        M = min(cpu_sample_paths(rate0, seconds / 2), 2_000_000_000)
        t0 = time.perf_counter()
        res = _cpu_run(mc_oracle, use_ref, model, p, M, nthreads)
        dt = time.perf_counter() - t0
        out[model] = {"paths_per_s": M / dt, "paths": M, "seconds": dt, "threads": nthreads,
                      "count": res["count"]}
    return kind, out


def _cpu_run(mc_oracle, use_ref, model, p, M, nthreads):
    os.environ["OMP_NUM_THREADS"] = str(nthreads)
    with quiet_stdout():
        if use_ref:
            return mc_oracle.ref_run(model, p.mu, p.sigma, M, p.k, p.x, p.seed, keep_upper=True,
                                     nthreads=nthreads)
        if model == "serial":
            return mc_oracle.serial_estimate(p.mu, p.sigma, M, p.k, p.x, p.seed, keep_upper=True)
        return mc_oracle.omp_estimate(p.mu, p.sigma, M, p.k, p.x, p.seed, keep_upper=True,
                                      nthreads=nthreads)


def reference_cuda_measure(steps):
    """The reference's own GPU kernel (src/05-GPU/monte_carlos_cuda.cu:23-72,
    compiled unmodified for sm_103a) timed on this GPU on the drop-in workload
    (N = 50, 1e8 paths, seed 67), launched as its host wrapper launches it,
    beside the engine's kernels on the same inputs: the reference's XORWOW
    layout (RG_RNG_XORWOW_REF, S per path stored as the reference stores it)
    and the engine's Philox fused kernel (counts only).  None where the
    reference kernel was not compiled (it needs the reference tree)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import mc_oracle
    if not mc_oracle.ref_kernel_available():
        return None
    import numpy as np
    import torch
    import riskgpu
    from riskgpu import synth
    M = 100_000_000
    p = synth.one_factor_50(n_paths=M)
    port = riskgpu.Portfolio(p.mu, p.sigma)
    L = np.ascontiguousarray(port.factor())
    d_mu = torch.tensor(p.mu, dtype=torch.float64, device="cuda")
    d_L = torch.tensor(L, dtype=torch.float64, device="cuda")
    S = torch.empty(M, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    ref_ms = []
    for i in range(steps + 1):
        ms = mc_oracle.ref_kernel_run(M, p.n, p.k, p.x, d_mu.data_ptr(), d_L.data_ptr(), p.seed, S.data_ptr(),
                                      cnt.data_ptr())
        if i:
            ref_ms.append(ms)
    ref_count = int(cnt.item())
    eng = {}
    for name, rng, dS in (("xorwow_layout_with_S", riskgpu.RNG_XORWOW_REF, S.data_ptr()),
                          ("philox_counts_only", riskgpu.RNG_PHILOX, None)):
        q = riskgpu.make_query(M, p.seed, x=p.x, k=p.k, horizon=1, port_threshold=-1.0, rng=rng,
                               precision=riskgpu.PREC_FP32, d_s_values=dS)
        port.simulate(q)
        ms = [port.simulate(q)["ms_device"] for _ in range(steps)]
        r = port.simulate(q)
        eng[name] = {"ms": sum(ms) / steps, "paths_per_s": M / (sum(ms) / steps * 1e-3),
                     "crash_count": r["crash_count"]}
    port.close()
    ref = sum(ref_ms) / steps
    return {"kernel": "monte_carlo_kernel (reference, unmodified, sm_103a)", "n_assets": p.n, "paths": M,
            "ms": ref, "paths_per_s": M / (ref * 1e-3), "crash_count": ref_count, "steps": steps,
            "engine": eng, "engine_xorwow_speedup": ref / eng["xorwow_layout_with_S"]["ms"],
            "engine_philox_speedup": ref / eng["philox_counts_only"]["ms"]}


def reference_arm(args):
    """The reference's CPU models on bounded samples of the workload's inputs:
    the warm-up steps calibrate both models (serial on 1 core, OpenMP on all
    host cores) and pick the faster; each timed step then runs one sample of
    about cpu_seconds / steps of work with it, and ms_per_step is that
    sample's measured time."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import mc_oracle
    mc_oracle.build()
    use_ref = mc_oracle.ref_available()
    kind = "reference" if use_ref else "port"
    p = workload(args)
    threads = os.cpu_count() or 1
    per_step = max(0.5, args.cpu_seconds / max(1, args.steps))
    rates = {}
    sizes = {"serial": 2000 if p.n <= 64 else 100, "openmp": 2000 if p.n <= 64 else 100}
    for i in range(max(2, args.warmup)):
        # each warm-up sizes the next sample from the rate just measured (a
        # call includes the model's own Cholesky, so small samples understate
        # the rate)
        for model, nthreads in (("serial", 1), ("openmp", threads)):
            t0 = time.perf_counter()
            _cpu_run(mc_oracle, use_ref, model, p, sizes[model], nthreads)
            rates[model] = (sizes[model] / max(time.perf_counter() - t0, 1e-6), nthreads)
            sizes[model] = cpu_sample_paths(rates[model][0], per_step / 2)
    best = max(rates, key=lambda m: rates[m][0])
    nthreads = rates[best][1]
    M = cpu_sample_paths(rates[best][0], per_step)
    step_s = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _cpu_run(mc_oracle, use_ref, best, p, M, nthreads)
        step_s.append(time.perf_counter() - t0)
    total = sum(step_s)
    value = M * args.steps / total
    sample = (f"{M} paths of the {args.workload} inputs per step with the reference's {best} model "
              f"({nthreads} threads; the reference's model has 1-day paths: N normals and a full N x N "
              f"dgemv each); warm-up rates: serial {rates['serial'][0]:.4g} paths/s, openmp "
              f"{rates['openmp'][0]:.4g} paths/s")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total / args.steps,
            "ms_per_step_basis": "measured: each step is one bounded sample of the workload",
            "sample_paths_per_step": M,
            "ms_per_full_step_extrapolated": 1e3 * args.paths / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config(args, world, p),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ oracle figures
def oracle_figures(name, p):
    """The FP64 oracle's figures for this workload's inputs, or None (with the
    reason) when the committed figures belong to other inputs."""
    import numpy as np
    try:
        with open(ORACLE_FIGURES) as f:
            figs = json.load(f)
    except OSError as e:
        return None, f"no oracle figures: {e}"
    fig = figs.get(name)
    if fig is None:
        return None, f"no oracle figures for {name}"
    h = hashlib.sha256()
    for a in (p.mu, p.sigma, p.weights):
        h.update(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    if h.hexdigest() != fig["inputs_sha256"]:
        return None, "the synthetic inputs differ from those of the oracle figures (numpy stream changed)"
    if (fig["x"], fig["k"], fig["horizon"], fig["port_threshold"]) != (p.x, p.k, p.horizon, p.port_threshold):
        return None, "the oracle figures were made for other thresholds or horizon"
    return fig, None


def se_units(r, fig, M):
    """(estimate - FP64 oracle) / standard error for one result dict."""
    out = {}
    pb = fig["p_breach"]
    out["p_breach"] = (r["p_breach"] - pb) / math.sqrt(pb * (1 - pb) / M)
    pc, pcs = fig["p_crash"], fig["p_crash_se"]
    # the oracle's own error (randomised QMC) is added in quadrature
    out["p_crash"] = (r["p_crash"] - pc) / math.sqrt(pc * (1 - pc) / M + pcs * pcs)
    if r.get("var") is not None and not math.isnan(r["var"]):
        se_q = math.sqrt(ALPHA * (1 - ALPHA) / M) / fig["density_at_var"]
        out["var"] = (r["var"] - fig["var"]) / se_q
        se_cv = math.sqrt(fig["excess_var"] / M) / (1 - ALPHA)
        out["cvar"] = (r["cvar"] - fig["cvar"]) / se_cv
    out["max_abs"] = max(abs(v) for v in out.values())
    return {k: round(v, 3) for k, v in out.items()}


# ------------------------------------------------------------------ timing
def pinned(a):
    """A numpy view of a page-locked copy of `a` (the end-to-end legs upload
    their inputs from pinned host memory)."""
    import numpy as np
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).pin_memory().numpy()


def time_steps(port, q, counts, stream, flush, steps, warmup):
    """W untimed launches, then K launches each bracketed by CUDA events on
    the launching stream, L2 flushed before each outside the events.
    Returns (per-step ms, (crash, breach) of the last step)."""
    import torch
    sp = stream.cuda_stream
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            port.launch_counts(q, counts.data_ptr(), sp)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        for i in range(steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            port.launch_counts(q, counts.data_ptr(), sp)
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev], tuple(int(v) for v in counts.cpu().tolist())


def served_measure(seconds, precision):
    """Poisson arrivals at 2000 queries/s, each a 1e5-path query on one of 64
    recurring portfolios drawn as in batch_256, through the server
    (continuous batching); against per-query launches of the plain kernel."""
    import numpy as np
    import riskgpu
    from riskgpu import synth
    ps = synth.batch_256(count=64, base_seed=5150)
    ports = [riskgpu.Portfolio(p.mu, p.sigma, p.weights) for p in ps]
    rng = np.random.default_rng(2000)
    rate = 2000.0
    nq = int(rate * seconds)
    picks = rng.integers(0, 64, nq)
    gaps = rng.exponential(1.0 / rate, nq)

    def query(j, prec):
        i = picks[j]
        return riskgpu.make_query(100_000, int(ps[i].seed) + j, x=ps[i].x, k=ps[i].k, horizon=ps[i].horizon,
                                  port_threshold=ps[i].port_threshold, precision=prec)
    queries = [query(j, precision) for j in range(nq)]
    srv = riskgpu.Server(slots=3, max_batch_items=64, poll_us=20)
    for i, pt in enumerate(ports):
        srv.register(i, pt)
    for t in [srv.submit(int(picks[j]), queries[j]) for j in range(min(64, nq))]:
        srv.wait(t)
    srv.reset_stats()
    # no Python garbage collection inside the arrival loop: a collected
    # engine handle frees device memory, which synchronises the device
    import gc
    gc.collect()
    gc.disable()
    t0 = time.perf_counter()
    tickets = []
    next_t = t0
    for j in range(nq):
        next_t += gaps[j]
        while time.perf_counter() < next_t:
            pass
        tickets.append(srv.submit(int(picks[j]), queries[j]))
    served = [srv.wait(t) for t in tickets]
    wall = time.perf_counter() - t0
    gc.enable()
    st = srv.stats()
    srv.close()
    # where the latency tail sits: percentiles from each result's own
    # submit-to-completion time, and when the slow queries were submitted
    lat_all = np.array([r["latency_ms"] for r in served])
    submit_s = np.cumsum(gaps)
    slow = np.nonzero(lat_all > 10.0)[0]
    tail = {"p90": float(np.percentile(lat_all, 90)), "p95": float(np.percentile(lat_all, 95)),
            "p999": float(np.percentile(lat_all, 99.9)), "over_10ms": int(slow.size),
            "slow_submit_s": [round(float(submit_s[j]), 4) for j in slow[:12]],
            "slow_shapes": [(int(ps[picks[j]].n), int(ps[picks[j]].horizon)) for j in slow[:12]]}
    # each result is the same as the query run alone (first 32)
    same = all(served[j]["crash_count"] == ports[picks[j]].simulate(queries[j])["crash_count"] and
               served[j]["breach_count"] == ports[picks[j]].simulate(queries[j])["breach_count"]
               for j in range(min(32, nq)))
    # per-query launches of the plain kernel, one at a time
    lat = []
    t1 = time.perf_counter()
    nplain = min(nq, 400)
    for j in range(nplain):
        s = time.perf_counter()
        ports[picks[j]].simulate(query(j, riskgpu.PREC_FP32))
        lat.append(1e3 * (time.perf_counter() - s))
    plain_s = time.perf_counter() - t1
    lat.sort()
    for pt in ports:
        pt.close()
    return {"arrivals": "Poisson 2000/s", "queries": nq, "paths_per_query": 100_000, "portfolios": 64,
            "precision": {riskgpu.PREC_BF16X3: "bf16x3", riskgpu.PREC_FP16X3: "fp16x3"}.get(precision, "fp32"),
            "offered_paths_per_s": rate * 1e5, "paths_per_s": st["paths_per_s"],
            "latency_ms": {"p50": st["p50_ms"], "p99": st["p99_ms"], "max": st["max_ms"]},
            "p99_under_10ms": st["p99_ms"] < 10.0, "latency_tail": tail, "wall_s": wall,
            "results_equal_alone_first32": same,
            "per_query_plain_fp32": {"queries": nplain, "queries_per_s": nplain / plain_s,
                                     "paths_per_s": nplain * 1e5 / plain_s,
                                     "service_p50_ms": lat[len(lat) // 2],
                                     "service_p99_ms": lat[max(0, int(0.99 * len(lat)) - 1)]},
            "server": {k: st[k] for k in st if k not in ("p50_ms", "p99_ms", "max_ms")}}


def batch_measure(steps, warmup, precision):
    """256 portfolios in one persistent tensor-core launch replayed from a
    CUDA graph; per-portfolio launches of the plain FP32 kernel and of the
    tensor-core kernel (device time) beside it."""
    import torch
    import riskgpu
    from riskgpu import synth
    ps = synth.batch_256()
    ports = [riskgpu.Portfolio(p.mu, p.sigma, p.weights) for p in ps]

    def q(p, prec):
        return riskgpu.make_query(p.n_paths, p.seed, x=p.x, k=p.k, horizon=p.horizon,
                                  port_threshold=p.port_threshold, precision=prec)
    total = sum(p.n_paths for p in ps)
    batch = riskgpu.Batch([(pt, q(p, precision)) for pt, p in zip(ports, ps)])
    batch.run()
    batch.tune()
    for _ in range(warmup):
        batch.run()
    stream = torch.cuda.Stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for i in range(steps):
        ev[i][0].record(stream)
        batch.launch(stream.cuda_stream)
        ev[i][1].record(stream)
    res = batch.wait()
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / steps
    value = total / (ms * 1e-3)

    def per_item(prec):
        dev = 0.0
        for pt, p in zip(ports, ps):
            dev += pt.simulate(q(p, prec))["ms_device"]
        return total / (dev * 1e-3)
    plain_dev = per_item(riskgpu.PREC_FP32)
    tc_dev = per_item(precision)
    same = all(r["crash_count"] == pt.simulate(q(p, precision))["crash_count"]
               for r, pt, p in list(zip(res, ports, ps))[:16])
    info = batch.info()
    batch.close()
    for pt in ports:
        pt.close()
    return {"portfolios": len(ps), "paths_per_step": total, "n_assets": "U{10..600}",
            "horizon_days": "U{1..20}", "paths": "log-uniform [1e4, 1e6]",
            "launch": "one persistent tcgen05 launch, CUDA graph", "value": value, "unit": UNIT,
            "ms_per_step": ms, "steps": steps,
            "per_portfolio_plain_fp32_paths_per_s_device": plain_dev,
            "per_portfolio_tensor_paths_per_s_device": tc_dev,
            "ratio_vs_per_portfolio_plain_fp32": value / plain_dev,
            "results_equal_alone_first16": same, "batch": info}


def one_factor_50_measure(steps, warmup, flush, peaks, sm_mhz=None):
    """The drop-in workload on the plain fused FP32 kernel: device paths/s,
    its roofline, and end to end through get_cuda_model().run_model."""
    import torch
    import riskgpu
    from riskgpu import synth
    M = 100_000_000
    p = synth.one_factor_50(n_paths=M)
    port = riskgpu.Portfolio(p.mu, p.sigma, p.weights)
    stream = torch.cuda.Stream()
    counts = torch.zeros(2, dtype=torch.int64, device="cuda")
    q = riskgpu.make_query(M, p.seed, x=p.x, k=p.k, horizon=1, port_threshold=p.port_threshold,
                           precision=riskgpu.PREC_FP32)
    step_ms, (crash, breach) = time_steps(port, q, counts, stream, flush, steps, warmup)
    ms = sum(step_ms) / steps
    n = p.n
    flops = n * (n + 1) + 2 * n
    normals = 4 * ((n + 3) // 4)
    achieved = flops * M / (ms * 1e-3) / 1e12
    t_ideal = (flops / (peaks["fp32_tflops"] * 1e12) + normals / peaks["normals_per_s"]) * M
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = sm_mhz or 2070.0
    issue_bound = sms * 128 * mhz * 1e6 / ROWS_THREAD_INST_PER_PATH
    r = port.simulate(riskgpu.make_query(M, p.seed, x=p.x, k=p.k, horizon=1, port_threshold=p.port_threshold,
                                         precision=riskgpu.PREC_FP32, var_level=ALPHA))
    port.close()
    fig, why = oracle_figures("one_factor_50", p)
    # end to end through the reference-facing plugin call (host mu, Sigma;
    # upload, factorisation, kernel and counts every call: cache off)
    os.environ["RG_PLUGIN_CACHE"] = "0"
    call = riskgpu.PluginCall(pinned(p.mu), pinned(p.sigma))
    with quiet_stdout():
        call.run(M, p.k, p.x, p.seed)
        t0 = time.perf_counter()
        for _ in range(3):
            if call.run(M, p.k, p.x, p.seed)["status"] != 0:
                raise RuntimeError("plugin call failed")
        e2e_s = (time.perf_counter() - t0) / 3
    return {"kernel": "rg::mc_rows_kernel<13,true,false>", "n_assets": n, "horizon_days": 1,
            "paths_per_step": M, "value": M / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "steps": steps,
            "roofline": {"bound": "alu", "achieved": achieved, "peak": peaks["fp32_tflops"], "unit": "TFLOP/s",
                         "frac": achieved / peaks["fp32_tflops"],
                         "composite_frac": t_ideal / (ms * 1e-3),
                         "issue_bound": {"paths_per_s": issue_bound, "frac": M / (ms * 1e-3) / issue_bound,
                                         "basis": f"{ROWS_THREAD_INST_PER_PATH} thread instructions per path (ncu) "
                                                  f"at 128 a cycle on each of {sms} SMs, {mhz:.0f} MHz"},
                         "traffic": NCU_TRAFFIC_BYTES["one_factor_50"]},
            "counts": {"crash": crash, "breach": breach},
            "se_units": se_units(r, fig, M) if fig else why,
            "e2e": {"value": M / e2e_s, "unit": UNIT, "ms_per_step": 1e3 * e2e_s,
                    "path": "get_cuda_model().run_model (host mu/Sigma)",
                    "h2d_bytes_per_step": 8 * n + 8 * n * n, "d2h_bytes_per_step": 16 + 4 + 16}}


# ------------------------------------------------------------------ engine arm
def engine_arm(args):
    import torch
    import riskgpu

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    p = workload(args)
    prec_name = precision_name(args)
    code = {"fp32": riskgpu.PREC_FP32, "bf16x3": riskgpu.PREC_BF16X3, "fp16x3": riskgpu.PREC_FP16X3}
    prec = code[prec_name]
    tensor = prec_name != "fp32"
    stream = torch.cuda.Stream()
    port = riskgpu.Portfolio(p.mu, p.sigma, p.weights)
    counts = torch.zeros(2, dtype=torch.int64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    draws = riskgpu.DRAWS_AGGREGATED if args.draw_mode == "aggregated" else riskgpu.DRAWS_DAILY
    # shard: rank r owns paths [r*M, (r+1)*M)
    offset, count = riskgpu.shard_range(rank, world, args.paths)

    def q_of(pr, dm=draws, var_level=0.0, n_paths=count, path_offset=offset):
        return riskgpu.make_query(n_paths, p.seed, x=p.x, k=p.k, horizon=p.horizon,
                                  port_threshold=p.port_threshold, path_offset=path_offset,
                                  precision=pr, draw_mode=dm, var_level=var_level)

    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    step_ms, (crash, breach) = time_steps(port, q_of(prec), counts, stream, flush, args.steps, args.warmup)
    barrier()
    wall = time.perf_counter() - wall0
    forms = {}
    if tensor:
        # the plain FP32 kernel on the same draws: the denominator of the metric
        for name in ("fp32", "fp16x3" if prec_name == "bf16x3" else "bf16x3"):
            ms_f, c_f = time_steps(port, q_of(code[name]), counts, stream, flush, args.steps, args.warmup)
            forms[name] = {"step_ms": ms_f, "counts": c_f}
    clk = clocks.stop()

    total_ms = sum(step_ms)
    tot = torch.tensor([total_ms] + [sum(f["step_ms"]) for f in forms.values()], device="cuda",
                       dtype=torch.float64)
    cnt = torch.tensor([crash, breach], device="cuda", dtype=torch.int64)
    if dist is not None:
        # the one exchange of the sharded path: the int64 counts are summed;
        # the timing is the max over ranks
        dist.all_reduce(tot, op=dist.ReduceOp.MAX)
        dist.all_reduce(cnt, op=dist.ReduceOp.SUM)
    tot = tot.cpu().tolist()
    crash_all, breach_all = [int(v) for v in cnt.cpu().tolist()]
    total_ms = tot[0]
    value = world * count * args.steps / (total_ms * 1e-3)
    ms_per_step = total_ms / args.steps
    for i, name in enumerate(forms):
        forms[name]["value"] = world * count * args.steps / (tot[1 + i] * 1e-3)
        forms[name]["ms_per_step"] = tot[1 + i] / args.steps

    peaks = riskgpu.probe_peaks(stream.cuda_stream)
    torch.cuda.synchronize()
    mp = measured_peaks()
    n = p.n
    flops_per_path = n * (n + 1) + 2 * n          # triangular contraction + w.R
    days = 1 if args.draw_mode == "aggregated" else p.horizon
    normals_per_path = n * days
    normals_drawn = 4 * ((n + 3) // 4) * days     # one Philox block per 4 assets and day
    normals_per_s = normals_drawn * count / (ms_per_step * 1e-3)
    tflops = flops_per_path * count / (ms_per_step * 1e-3) / 1e12
    key = "five_factor_600" if n == 600 else args.workload
    if tensor:
        # with daily draws the normal generation on the ALU/XU pipes bounds the
        # tcgen05 form; the contraction's tensor-pipe rate is beside it
        roofline = {"bound": "alu", "kernel": "rg::mc_tcws_kernel<false,false,96>",
                    "achieved": normals_per_s, "peak": peaks["normals_per_s"], "unit": "normals/s",
                    "frac": normals_per_s / peaks["normals_per_s"],
                    "peak_source": "measured live: Philox4x32-10 + Box-Muller micro-kernel (rg_probe_peaks)",
                    "tensor": {"achieved_tflops": tflops, "peak_tflops": mp["bf16_tflops"],
                               "frac": tflops / mp["bf16_tflops"], "peak_source": mp["source"] + " BF16 burst",
                               "issued_tflops_dense_x3": 3 * 2 * n * n * count / (ms_per_step * 1e-3) / 1e12},
                    "algorithmic_flops_per_path": flops_per_path, "normals_per_path": normals_per_path,
                    "traffic": NCU_TRAFFIC_BYTES.get(key)}
        if n == 600 and args.draw_mode == "daily":
            sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
            mhz = clk.get("sm_mhz") or 2070.0
            bound = sms * 128 * mhz * 1e6 / TC_THREAD_INST_PER_NORMAL
            roofline["issue_bound"] = {
                "normals_per_s": bound, "frac": normals_per_s / bound,
                "basis": f"{TC_THREAD_INST_PER_NORMAL} thread instructions per normal (ncu) at 128 a cycle on "
                         f"each of {sms} SMs, {mhz:.0f} MHz"}
    else:
        t_ideal = (flops_per_path / (peaks["fp32_tflops"] * 1e12)
                   + normals_drawn / peaks["normals_per_s"]) * count
        roofline = {"bound": "alu",
                    "kernel": "rg::mc_rows_kernel<13,true,false>" if n <= 64 else "rg::mc_tiled_pipe_kernel<false,32>",
                    "achieved": tflops, "peak": peaks["fp32_tflops"], "unit": "TFLOP/s",
                    "frac": tflops / peaks["fp32_tflops"],
                    "peak_source": "measured live: FP32 FMA micro-kernel (rg_probe_peaks)",
                    "composite_frac": t_ideal / (ms_per_step * 1e-3),
                    "normals_per_s": normals_per_s, "normals_peak": peaks["normals_per_s"],
                    "algorithmic_flops_per_path": flops_per_path,
                    "traffic": NCU_TRAFFIC_BYTES.get(key)}
        if n == 50 and p.horizon == 1:
            sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
            mhz = clk.get("sm_mhz") or 2070.0
            bound = sms * 128 * mhz * 1e6 / ROWS_THREAD_INST_PER_PATH
            roofline["issue_bound"] = {
                "paths_per_s": bound, "frac": count / (ms_per_step * 1e-3) / bound,
                "basis": f"{ROWS_THREAD_INST_PER_PATH} thread instructions per path (ncu) at 128 a cycle on "
                         f"each of {sms} SMs, {mhz:.0f} MHz"}
    if "fp32" in forms:
        f = forms["fp32"]
        t_ideal = (flops_per_path / (peaks["fp32_tflops"] * 1e12)
                   + normals_drawn / peaks["normals_per_s"]) * count
        f["roofline"] = {"kernel": "rg::mc_tiled_pipe_kernel<false,32>",
                         "frac": flops_per_path * count / (f["ms_per_step"] * 1e-3) / (peaks["fp32_tflops"] * 1e12),
                         "composite_frac": t_ideal / (f["ms_per_step"] * 1e-3)}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp16x3": "f16x3", "bf16x3": "bf16x3"}.get(prec_name, "f32"), "data": "synthetic",
            "config": config(args, world, p)}
    if "fp32" in forms:
        line["plain_fp32"] = {k: v for k, v in forms["fp32"].items() if k != "step_ms"}
        line["ratio_vs_plain_fp32"] = value / forms["fp32"]["value"]
    for name in ("fp16x3", "bf16x3"):
        if name in forms:
            line[name] = {k: v for k, v in forms[name].items() if k != "step_ms"}
            line[name]["ratio_vs_plain_fp32"] = forms[name]["value"] / forms["fp32"]["value"]
    line["counts"] = {"crash": crash_all, "breach": breach_all, "paths": world * count}
    # the headline's timed region launches one kernel per step; the other
    # forms' timed regions launch one each per step too
    line["gpu_launches"] = args.steps
    line["gpu_launches_other_forms"] = args.steps * len(forms)
    line["clocks"] = clk
    line["roofline"] = roofline
    line["wall_s_timed_region"] = wall
    line["step_ms"] = [round(v, 4) for v in step_ms]

    if rank == 0 and world == 1:
        # ---- errors in Monte Carlo standard errors against the FP64 oracle,
        # every form, same paths (a VaR pass is added to the counting pass)
        fig, why = oracle_figures(key, p)
        if fig is not None:
            se = {}
            for name in [prec_name] + list(forms):
                r = port.simulate(q_of(code[name], var_level=ALPHA))
                se[name] = se_units(r, fig, count)
                se[name]["counts_match_timed_run"] = (
                    (r["crash_count"], r["breach_count"]) ==
                    ((crash, breach) if name == prec_name else tuple(forms[name]["counts"])))
            line["se_units"] = se
            line["se_units_all_within_3"] = all(v["max_abs"] <= 3.0 for v in se.values())
            line["oracle"] = {"p_crash": fig["p_crash"], "p_crash_se": fig["p_crash_se"],
                              "p_crash_method": fig["p_crash_method"], "p_breach": fig["p_breach"],
                              "var": fig["var"], "cvar": fig["cvar"], "alpha": ALPHA}
        else:
            line["se_units"] = why

        # ---- aggregated draws (one N(0, H) draw per asset: the same H-day
        # distribution, H times fewer normals), both forms
        if tensor and args.draw_mode == "daily" and not args.no_extras:
            agg = {}
            for name in (prec_name, "fp32"):
                ms_a, _ = time_steps(port, q_of(code[name], dm=riskgpu.DRAWS_AGGREGATED), counts, stream, flush,
                                     args.steps, args.warmup)
                agg[name] = {"value": count * args.steps / (sum(ms_a) * 1e-3), "ms_per_step": sum(ms_a) / args.steps}
            agg["ratio_vs_plain_fp32"] = agg[prec_name]["value"] / agg["fp32"]["value"]
            line["aggregated_draws"] = agg

        # ---- e2e through the public C ABI with host buffers: the plugin API
        # (get_cuda_model) has no horizon, weights or precision, so the
        # precision form goes through rg_run
        os.environ.pop("RG_MATERIALIZE_S", None)
        os.environ.pop("RG_RNG", None)
        if args.workload == "one_factor_50":
            os.environ["RG_PLUGIN_CACHE"] = "0"
            call = riskgpu.PluginCall(pinned(p.mu), pinned(p.sigma))
            run_once = lambda: call.run(count, p.k, p.x, p.seed)["status"] == 0 or sys.exit("plugin call failed")
            e2e_path = "get_cuda_model().run_model (host mu/Sigma: upload, GPU Cholesky, kernel, counts back)"
            h2d = 8 * n + 8 * n * n
        else:
            qh = q_of(prec)
            mu_h, sigma_h, w_h = pinned(p.mu), pinned(p.sigma), pinned(p.weights)
            run_once = lambda: riskgpu.run(mu_h, sigma_h, w_h, qh)
            e2e_path = "rg_run (host mu/Sigma/weights: upload, GPU Cholesky, tiles, kernel, counts back)"
            h2d = 8 * n + 8 * n * n + 8 * n
        with quiet_stdout():
            run_once()
            e2e_steps = max(3, min(args.steps, 5))
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                run_once()
            e2e_s = (time.perf_counter() - t0) / e2e_steps
        line["e2e"] = {"value": count / e2e_s, "unit": UNIT, "ms_per_step": 1e3 * e2e_s, "path": e2e_path,
                       "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 16 + 4 + 16}
        port.close()
        del flush
        torch.cuda.empty_cache()
        if not args.no_extras and args.workload == "five_factor_600":
            flush2 = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
            line["one_factor_50"] = one_factor_50_measure(min(args.steps, 20), args.warmup, flush2, peaks,
                                                          (line.get("clocks") or {}).get("sm_mhz"))
            del flush2
            line["batched"] = batch_measure(min(args.steps, 10), args.warmup, riskgpu.PREC_BF16X3)
            line["served"] = served_measure(1.0, riskgpu.PREC_BF16X3)
        if not args.no_cpu_baseline:
            # baselines: the reference's GPU kernel on this GPU, then its CPU
            # models on this host
            rc = reference_cuda_measure(3)
            line["reference_cuda"] = rc if rc is not None else "not compiled here (needs the reference tree)"
            kind, det = run_cpu_reference(p, args.cpu_seconds, os.cpu_count() or 1)
            s = det["serial"]
            line["cpu_baseline"] = {"value": s["paths_per_s"], "unit": UNIT, "cores": 1, "kind": kind,
                                    "sample": f"{s['paths']} paths of the {args.workload} inputs, reference "
                                              f"serial model (1-day paths: MT19937 + polar normals + FP64 "
                                              f"full dgemv), 1 thread",
                                    "openmp_all_cores": {"value": det["openmp"]["paths_per_s"],
                                                         "cores": det["openmp"]["threads"]}}
    else:
        port.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def batch_arm(args):
    import torch
    import riskgpu
    torch.cuda.set_device(0)
    clocks = ClockSampler(0)
    clocks.start()
    b = batch_measure(args.steps, args.warmup, riskgpu.PREC_BF16X3)
    clk = clocks.stop()
    line = {"metric": METRIC, "value": b["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": b["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16x3", "data": "synthetic",
            "config": {"workload": "batch_256"}, "batched": b, "clocks": clk, "gpu_launches": args.steps}
    print(json.dumps(line), flush=True)


def served_arm(args):
    import torch
    import riskgpu
    torch.cuda.set_device(0)
    clocks = ClockSampler(0)
    clocks.start()
    s = served_measure(max(1.0, float(args.steps) / 10.0), riskgpu.PREC_BF16X3)
    clk = clocks.stop()
    line = {"metric": "served_paths_per_second", "value": s["paths_per_s"], "unit": UNIT, "n_gpus": 1,
            "steps": s["queries"], "warmup": 64, "ms_per_step": 1e3 * s["wall_s"] / s["queries"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3",
            "data": "synthetic", "config": {"workload": "served"}, "served": s, "clocks": clk}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    elif args.workload == "batch_256":
        batch_arm(args)
    elif args.workload == "served":
        served_arm(args)
    else:
        engine_arm(args)


if __name__ == "__main__":
    main()

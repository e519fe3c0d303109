"""Benchmark: paths/s of the plain fused FP32 kernel on the drop-in workload.

Workload (the configuration the headline metric is quoted on):
  one_factor_50  N = 50 assets, one-factor covariance, 1-day horizon,
                 M = 1e8 paths per step, Dirichlet(1) weights, portfolio
                 threshold -3%, crash semantics x = 0.03, k = 5, seed 67,
                 Philox normals, FP32 returns, FP64 Cholesky (done once,
                 resident).  Synthetic inputs (numpy PCG64), no data set.

A step is one pass of the fused kernel over the M paths of the batch (the
breach and crash counts of every path, exact 64-bit integers).

`value`   paths/s with the factor resident in HBM, device time of the K timed
          kernels (CUDA events on the launching stream).  The kernel's inputs
          are a few KB, so L2 is flushed (a 256 MB write) before every timed
          step, outside the event pair.
`e2e`     paths/s through the reference-facing plugin call
          (get_cuda_model().run_model, host buffers): every step uploads mu and
          Sigma, factors on the GPU, runs the kernel and reads the counts back.
`roofline` the fused kernel against the measured FP32 FMA peak (rg_probe_peaks),
          plus the composite issue bound that also charges normal generation
          at the measured normal-generation peak.
`cpu_baseline` the oracle's restatement of the reference's C serial model on the
          host (1 core), bounded sample.

--impl reference times the reference's CPU implementation of this path (its
serial and OpenMP models; compiled from the reference's sources where the
reference tree exists, else the oracle's restatement of them) on all host
cores, on a bounded sample of the same workload.
"""
import argparse
import contextlib
import io
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

# DRAM bytes (read + write) per launch of the fused N=50 kernel from one ncu
# capture (profiles/mc_rows_one_factor_50.md: 41.2 KB + 1.3 KB; it does not
# grow with the paths per launch, only the factor and the counters move).
NCU_TRAFFIC_BYTES = 42_496


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="riskgpu", choices=["riskgpu", "reference"])
    ap.add_argument("--paths", type=int, default=None,
                    help="paths per step (default: the workload's, 1e8 or 1e7)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="approximate CPU time of the bounded CPU samples")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="one_factor_50",
                    choices=["one_factor_50", "five_factor_600", "batch_256", "served"],
                    help="one_factor_50 is the headline; five_factor_600 (N=600, H=10, "
                         "M=1e7 per step) is the precision-form workload")
    ap.add_argument("--draw-mode", default="daily", choices=["daily", "aggregated"])
    ap.add_argument("--precision", default="auto", choices=["auto", "fp32", "bf16x3", "fp16x3"])
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(args):
    """The synthetic portfolio of the workload, sized to the paths per step."""
    from riskgpu import synth
    if args.workload == "five_factor_600":
        if args.paths is None:
            args.paths = 10_000_000
        return synth.five_factor_600(n_paths=args.paths)
    if args.paths is None:
        args.paths = 100_000_000
    return synth.one_factor_50(n_paths=args.paths)


def config(args, world, p):
    return {"workload": args.workload, "n_assets": p.n, "horizon_days": p.horizon,
            "paths_per_step": args.paths,
            "factor": "one-factor" if p.n == 50 else "five-factor", "weights": "Dirichlet(1)",
            "port_threshold": p.port_threshold, "x": p.x, "k": p.k, "rng": "philox4x32-10",
            "draws": args.draw_mode, "precision": args.precision,
            "cholesky": "fp64 on GPU, resident", "l2": "flushed (256 MB write) before each timed step",
            "parallelism": f"path-range shards x{world}" if world > 1 else "1 GPU"}


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


def cpu_sample_paths(rate_guess, seconds):
    return max(2000, int(rate_guess * seconds))


def run_cpu_reference(p, seconds, threads):
    """The reference's CPU models on a bounded sample: (paths/s, details)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import mc_oracle
    mc_oracle.build()
    use_ref = mc_oracle.ref_available()
    kind = "reference" if use_ref else "port"
    out = {}
    for model, nthreads in (("serial", 1), ("openmp", threads)):
        # calibrate on a small sample, then run ~seconds of work
        M0 = 2000
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


def reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    p = workload(args)
    threads = os.cpu_count() or 1
    times, kinds, details = [], None, None
    # warm-up + K timed steps, each a bounded sample of the workload
    per_step = max(1.0, args.cpu_seconds / max(1, args.steps))
    for i in range(args.warmup + args.steps):
        kind, det = run_cpu_reference(p, per_step if i >= args.warmup else 0.5, threads)
        if i >= args.warmup:
            best = max(det.values(), key=lambda d: d["paths_per_s"])
            times.append(best["paths_per_s"])
            kinds, details = kind, det
    value = statistics.median(times)
    best_model = max(details, key=lambda m: details[m]["paths_per_s"])
    sample = (f"{details[best_model]['paths']} paths of the {args.workload} workload per step with the "
              f"reference's {best_model} model ({details[best_model]['threads']} threads); "
              f"serial {details['serial']['paths_per_s']:.4g} paths/s, openmp "
              f"{details['openmp']['paths_per_s']:.4g} paths/s")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            # the time one full step of args.paths would take at the measured
            # rate; each timed step ran the bounded sample below
            "ms_per_step": 1e3 * args.paths / value,
            "ms_per_step_basis": "extrapolated from bounded samples",
            "sample_paths_per_step": details[best_model]["paths"],
            "sample_ms_per_step": 1e3 * details[best_model]["paths"] / details[best_model]["paths_per_s"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config(args, world, p),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": details[best_model]["threads"],
                             "kind": kinds, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def engine_arm(args):
    import torch
    import riskgpu
    from riskgpu import synth

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
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    port = riskgpu.Portfolio(p.mu, p.sigma, p.weights)
    counts = torch.zeros(2, dtype=torch.int64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    # shard: rank r owns paths [r*M, (r+1)*M)
    prec = {"auto": riskgpu.PREC_AUTO, "fp32": riskgpu.PREC_FP32, "bf16x3": riskgpu.PREC_BF16X3,
            "fp16x3": riskgpu.PREC_FP16X3}[args.precision]
    draws = riskgpu.DRAWS_AGGREGATED if args.draw_mode == "aggregated" else riskgpu.DRAWS_DAILY
    offset, count = riskgpu.shard_range(rank, world, args.paths)
    q = riskgpu.make_query(count, p.seed, x=p.x, k=p.k, horizon=p.horizon,
                           port_threshold=p.port_threshold, path_offset=offset,
                           precision=prec, draw_mode=draws)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            port.launch_counts(q, counts.data_ptr(), sp)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        clocks = ClockSampler(torch.cuda.current_device())
        clocks.start()
        barrier()
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        results = []
        for i in range(args.steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            port.launch_counts(q, counts.data_ptr(), sp)
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        barrier()
        wall = time.perf_counter() - wall0
        clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)
    crash, breach = [int(v) for v in counts.cpu().tolist()]
    if dist is not None:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * args.paths * args.steps / (total_ms * 1e-3)
    ms_per_step = total_ms / args.steps

    # ---- e2e through the reference-facing plugin call (host buffers); the
    # plugin API has no horizon or weights, so other workloads go through
    # rg_run (host mu, Sigma, weights; the same copies, factorisation and
    # kernel)
    e2e_steps = max(3, min(args.steps, 5))
    os.environ.pop("RG_MATERIALIZE_S", None)
    os.environ.pop("RG_RNG", None)
    # every step uploads and factors its inputs: the plugin path's cache of
    # resident factors is off for this measurement
    os.environ["RG_PLUGIN_CACHE"] = "0"
    if args.workload == "one_factor_50":
        call = riskgpu.PluginCall(p.mu, p.sigma)
        run_once = lambda: call.run(args.paths, p.k, p.x, p.seed)["status"]
        e2e_path = "get_cuda_model().run_model (host mu/Sigma)"
    else:
        qh = riskgpu.make_query(args.paths, p.seed, x=p.x, k=p.k, horizon=p.horizon,
                                port_threshold=p.port_threshold, precision=prec, draw_mode=draws)
        run_once = lambda: (riskgpu.run(p.mu, p.sigma, p.weights, qh), 0)[1]
        e2e_path = "rg_run (host mu/Sigma/weights)"
    with quiet_stdout():
        run_once()  # warm-up
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            if run_once() != 0:
                raise RuntimeError("end-to-end call failed")
        barrier()
        e2e_s = (time.perf_counter() - t0) / e2e_steps
    h2d = 8 * p.n + 8 * p.n * p.n + (8 * p.n if args.workload != "one_factor_50" else 0)
    d2h = 16 + 4 + 16  # counts, Cholesky info, portfolio moments

    # ---- roofline of the fused kernel
    peaks = riskgpu.probe_peaks(sp)
    torch.cuda.synchronize()
    n = p.n
    flops_per_path = n * (n + 1) + 2 * n          # triangular contraction + w.R
    days = 1 if args.draw_mode == "aggregated" else p.horizon
    normals_per_path = 4 * ((n + 3) // 4) * days   # one Philox block per 4 assets and day
    achieved = flops_per_path * args.paths / (ms_per_step * 1e-3) / 1e12
    t_ideal = (flops_per_path / (peaks["fp32_tflops"] * 1e12)
               + normals_per_path / peaks["normals_per_s"]) * args.paths
    normals_per_s = normals_per_path * args.paths / (ms_per_step * 1e-3)
    if prec in (riskgpu.PREC_FP16X3, riskgpu.PREC_BF16X3):
        # tcgen05 form: the contraction runs on the tensor pipe (three split
        # products); what bounds it is the normal generation on the ALU/XU
        # pipes, so the roofline is normals/s against the measured generator
        # peak, with the tensor-pipe rate beside it
        kname = "rg::mc_tcws_kernel<false,false>"
        roofline = {"bound": "alu", "kernel": kname,
                    "achieved": normals_per_s, "peak": peaks["normals_per_s"], "unit": "normals/s",
                    "frac": normals_per_s / peaks["normals_per_s"],
                    "peak_source": "measured live: Philox4x32-10 + Box-Muller micro-kernel (rg_probe_peaks)",
                    "tensor_tflops_useful_x3": 3 * achieved,
                    "algorithmic_flops_per_path": flops_per_path,
                    "normals_per_path": normals_per_path,
                    "traffic": None}
    else:
        kname = ("rg::mc_rows_kernel<13,true,false> (N=50)" if n <= 64 else "rg::mc_tiled_kernel<false>")
        roofline = {"bound": "alu", "kernel": kname,
                    "achieved": achieved, "peak": peaks["fp32_tflops"], "unit": "TFLOP/s",
                    "frac": achieved / peaks["fp32_tflops"],
                    "peak_source": "measured live: FP32 FMA micro-kernel (rg_probe_peaks)",
                    "composite_frac": t_ideal / (ms_per_step * 1e-3),
                    "normals_per_s": normals_per_s,
                    "normals_peak": peaks["normals_per_s"],
                    "algorithmic_flops_per_path": flops_per_path,
                    "traffic": NCU_TRAFFIC_BYTES if n <= 64 else None}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp16x3": "f16x3", "bf16x3": "bf16x3"}.get(args.precision, "f32"), "data": "synthetic",
            "config": config(args, world, p),
            "e2e": {"value": world * args.paths / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_s, "path": e2e_path},
            "gpu_launches": args.steps, "clocks": clk, "roofline": roofline,
            "wall_s_timed_region": wall, "counts_last_step": {"crash": crash, "breach": breach},
            "step_ms": [round(v, 4) for v in step_ms]}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        kind, det = run_cpu_reference(p, args.cpu_seconds, os.cpu_count() or 1)
        s = det["serial"]
        line["cpu_baseline"] = {"value": s["paths_per_s"], "unit": UNIT, "cores": 1, "kind": kind,
                                "sample": f"{s['paths']} paths of {args.workload}, reference serial model "
                                          f"(MT19937 + polar normals + FP64 dgemv), 1 thread",
                                "openmp_all_cores": {"value": det["openmp"]["paths_per_s"],
                                                     "cores": det["openmp"]["threads"]}}
    if rank == 0:
        print(json.dumps(line), flush=True)
    port.close()
    if dist is not None:
        dist.destroy_process_group()


def batch_arm(args):
    """256 portfolios (N ~ U{10..600}, H ~ U{1..20}, M log-uniform [1e4, 1e6],
    3-factor covariance, per-portfolio seed, thresholds U(-5%, -1%)) in one
    persistent tensor-core launch replayed from a CUDA graph, against
    per-portfolio launches of the plain FP32 kernels and of the tensor-core
    kernel."""
    import torch
    import riskgpu
    from riskgpu import synth
    torch.cuda.set_device(0)
    ps = synth.batch_256()
    ports = [riskgpu.Portfolio(p.mu, p.sigma, p.weights) for p in ps]

    def q(p, prec):
        return riskgpu.make_query(p.n_paths, p.seed, x=p.x, k=p.k, horizon=p.horizon,
                                  port_threshold=p.port_threshold, precision=prec)
    total = sum(p.n_paths for p in ps)
    batch = riskgpu.Batch([(pt, q(p, riskgpu.PREC_FP16X3)) for pt, p in zip(ports, ps)])
    batch.run()
    batch.tune()
    for _ in range(args.warmup):
        batch.run()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stream = torch.cuda.Stream()
    clocks = ClockSampler(0)
    clocks.start()
    torch.cuda.synchronize()
    for i in range(args.steps):
        ev[i][0].record(stream)
        batch.launch(stream.cuda_stream)
        ev[i][1].record(stream)
    res = batch.wait()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    value = total / (ms * 1e-3)
    # per-portfolio launches, device-timed, same queries
    def per_item(prec):
        t0 = time.perf_counter()
        dev = 0.0
        for pt, p in zip(ports, ps):
            dev += pt.simulate(q(p, prec))["ms_device"]
        return total / (time.perf_counter() - t0), total / (dev * 1e-3)
    plain_wall, plain_dev = per_item(riskgpu.PREC_FP32)
    tc_wall, tc_dev = per_item(riskgpu.PREC_FP16X3)
    same = all(r["crash_count"] == pt.simulate(q(p, riskgpu.PREC_FP16X3))["crash_count"]
               for r, pt, p in list(zip(res, ports, ps))[:16])
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f16x3", "data": "synthetic",
            "config": {"workload": "batch_256", "portfolios": len(ps), "paths_per_step": total,
                       "n_assets": "U{10..600}", "horizon_days": "U{1..20}",
                       "paths": "log-uniform [1e4, 1e6]", "launch": "one persistent tcgen05 launch, CUDA graph",
                       "batch": batch.info()},
            "per_portfolio_launches": {"plain_fp32_paths_per_s_wall": plain_wall,
                                       "plain_fp32_paths_per_s_device": plain_dev,
                                       "tensor_paths_per_s_wall": tc_wall,
                                       "tensor_paths_per_s_device": tc_dev,
                                       "batched_over_plain_device": value / plain_dev},
            "results_equal_alone_first16": same, "clocks": clk, "gpu_launches": args.steps}
    print(json.dumps(line), flush=True)


def served_arm(args):
    """Poisson arrivals at 2000 queries/s, each a 64-recurring-portfolio
    query drawn as in batch_256 with M = 1e5, through the server (continuous
    batching); against per-query launches of the plain FP32 kernel."""
    import torch
    import numpy as np
    import riskgpu
    from riskgpu import synth
    torch.cuda.set_device(0)
    ps = synth.batch_256(count=64, base_seed=5150)
    ports = [riskgpu.Portfolio(p.mu, p.sigma, p.weights) for p in ps]
    rng = np.random.default_rng(2000)
    rate, seconds = 2000.0, max(1.0, float(args.steps) / 10.0)
    nq = int(rate * seconds)
    picks = rng.integers(0, 64, nq)
    gaps = rng.exponential(1.0 / rate, nq)
    queries = [riskgpu.make_query(100_000, int(ps[i].seed) + j, x=ps[i].x, k=ps[i].k, horizon=ps[i].horizon,
                                  port_threshold=ps[i].port_threshold, precision=riskgpu.PREC_FP16X3)
               for j, i in enumerate(picks)]
    srv = riskgpu.Server(slots=3, max_batch_items=64, poll_us=20)
    for i, pt in enumerate(ports):
        srv.register(i, pt)
    # warm-up
    for t in [srv.submit(int(picks[j]), queries[j]) for j in range(64)]:
        srv.wait(t)
    srv.reset_stats()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    tickets = []
    next_t = t0
    for j in range(nq):
        next_t += gaps[j]
        while time.perf_counter() < next_t:
            pass
        tickets.append(srv.submit(int(picks[j]), queries[j]))
    for t in tickets:
        srv.wait(t)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    # per-query launches of the plain kernel, one at a time
    lat = []
    t1 = time.perf_counter()
    for j in range(min(nq, 400)):
        s = time.perf_counter()
        qq = queries[j]
        qq.precision = riskgpu.PREC_FP32
        ports[picks[j]].simulate(qq)
        lat.append(1e3 * (time.perf_counter() - s))
    plain_s = time.perf_counter() - t1
    lat.sort()
    line = {"metric": "served_paths_per_second", "value": st["paths_per_s"], "unit": UNIT, "n_gpus": 1,
            "steps": nq, "warmup": 64, "ms_per_step": 1e3 * wall / nq, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f16x3", "data": "synthetic",
            "config": {"workload": "served", "arrivals": "Poisson 2000/s", "queries": nq,
                       "paths_per_query": 100_000, "portfolios": 64, "offered_paths_per_s": rate * 1e5},
            "latency_ms": {"p50": st["p50_ms"], "p99": st["p99_ms"], "max": st["max_ms"]},
            "server": st, "wall_s": wall,
            "per_query_plain": {"queries": len(lat), "queries_per_s": len(lat) / plain_s,
                                "paths_per_s": len(lat) * 1e5 / plain_s,
                                "service_p50_ms": lat[len(lat) // 2], "service_p99_ms": lat[int(0.99 * len(lat)) - 1]},
            "clocks": clk}
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

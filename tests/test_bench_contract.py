"""The reference arm of bench.py (CPU only): one JSON line with the keys the
benchmark contract names, on a bounded sample of the headline workload."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--cpu-seconds", "0.5"], capture_output=True, text=True, cwd=ROOT,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["metric"] == "paths_per_second" and d["unit"] == "paths/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["workload"] == "five_factor_600" and d["config"]["n_assets"] == 600
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"]
    assert d["sample_paths_per_step"] > 0 and d["ms_per_step_basis"].startswith("measured")
    assert d["ms_per_full_step_extrapolated"] > 0


def test_horizon_override_changes_only_the_horizon():
    """--horizon (instruction-count sweeps) replaces five_factor_600's 10-day
    horizon and nothing else; values below one day are refused."""
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "gpu-montecarlo-risk_gb300"))
    import importlib
    bench = importlib.import_module("bench")
    argv = sys.argv
    try:
        sys.argv = ["bench.py", "--paths", "1000"]
        base = bench.workload(bench.parse())
        sys.argv = ["bench.py", "--paths", "1000", "--horizon", "2"]
        args = bench.parse()
        p = bench.workload(args)
        assert base.horizon == 10 and p.horizon == 2
        assert p.n == base.n and p.k == base.k and p.x == base.x and p.seed == base.seed
        assert (p.mu == base.mu).all() and (p.sigma == base.sigma).all()
        assert bench.config(args, 1, p)["horizon_days"] == 2
        sys.argv = ["bench.py", "--paths", "1000", "--horizon", "0"]
        try:
            bench.workload(bench.parse())
        except SystemExit:
            pass
        else:
            raise AssertionError("--horizon 0 was accepted")
        sys.argv = ["bench.py", "--workload", "one_factor_50", "--paths", "1000", "--horizon", "2"]
        try:
            bench.workload(bench.parse())
        except SystemExit:
            pass
        else:
            raise AssertionError("--horizon was accepted for one_factor_50")
    finally:
        sys.argv = argv

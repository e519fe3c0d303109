"""The drop-in, proven with the reference's own host program.

src/main_runner.c, src/utilities/load_binary.c, src/utilities/csv_writer.c
and the reference's serial model are compiled unchanged with -DCUDA_BUILD
-DSERIAL_BUILD (oracle/Makefile, target refhost; the reference's Makefile
does the same at Makefile:60-72) and linked against the engine's
libriskgpu.so, which supplies get_cuda_model (main_runner.c:24-26,230-236).
Only the libyaml config loader is replaced by a test stand-in with its
interface (oracle/load_config_stub.c).

The program reads data/mu.bin, data/sigma.bin, data/params.bin (written in
the reference's binary format) and config.yaml from its working directory,
asks for a comment on stdin (given /dev/null), runs the listed models and
appends to results/simulation_results.csv.

Without a GPU the engine's model must be called and fail cleanly (return -1
with its message, main_runner carrying on with the next model); with a GPU
its printed count must equal rg_run's for the same inputs.  Built where the
reference tree is present; skipped elsewhere.
"""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference"
RUNNER = os.path.join(ROOT, "oracle", "_ref", "ref_main_runner")


@pytest.fixture(scope="module")
def runner(engine):
    if not os.path.isdir(os.path.join(REF, "src")):
        pytest.skip("the reference tree is not present")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "refhost"], check=True)
    return RUNNER


def _run(runner, tmp_path, models, M=20_000):
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=M)
    synth.write_reference_bins(p, str(tmp_path / "data"), actual_freq=0.0125)
    (tmp_path / "results").mkdir()
    (tmp_path / "config.yaml").write_text(
        "models:\n" + "".join(f"  - {m}\n" for m in models) +
        'start: "2015-01-01"\nend: "2025-12-31"\nindices:\n  AEX: "AEX.csv"\n'
        f"train_ratio: 0.8\nM: {M}\nrandom_seed: {p.seed}\nx: {p.x}\nk: {p.k}\ncomment: \"drop-in test\"\n")
    with open(os.devnull) as null:
        r = subprocess.run([runner], cwd=tmp_path, stdin=null, capture_output=True, text=True, timeout=300)
    return p, r


def _count(out, name):
    m = re.search(rf"{name} RESULTS\nEstimated Probability \(P_MIN\): ([0-9.]+)\n"
                  rf"Extreme Events Count: (\d+) out of (\d+) trials", out)
    return (float(m.group(1)), int(m.group(2)), int(m.group(3))) if m else None


def test_reference_host_calls_the_drop_in(runner, tmp_path, engine):
    p, r = _run(runner, tmp_path, ["serial", "cuda"])
    assert r.returncode == 0, r.stderr[-2000:]
    out = r.stdout
    # the reference's own serial model ran through the same host
    serial = _count(out, "serial")
    assert serial is not None and serial[2] == 20_000
    # main_runner selected get_cuda_model() and called run_model: the
    # engine's cuda_simulate printed its start line (.cu:76)
    assert "=== Running cuda model ===" in out
    assert "Starting CUDA Monte Carlo simulation with M = 20000 trials..." in out
    if engine.lib().rg_device_count() < 1:
        # no device: run_model returned -1 with the engine's message and the
        # host reported the failure and went on
        assert "no CUDA device" in r.stderr
        assert "Error: cuda model failed" in r.stderr
        assert _count(out, "cuda") is None
    else:
        cuda = _count(out, "cuda")
        assert cuda is not None
        q = engine.make_query(20_000, p.seed, x=p.x, k=p.k, horizon=1, port_threshold=0.0)
        res = engine.run(p.mu, p.sigma, None, q)
        assert cuda[1] == res["crash_count"]
    # the host wrote its CSV row for the serial model
    csv = (tmp_path / "results" / "simulation_results.csv").read_text()
    assert "serial" in csv
    assert "Simulation complete." in out

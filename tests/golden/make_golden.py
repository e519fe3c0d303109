"""Generate the golden vectors under tests/golden/ from the reference itself.

Run in a tree where the reference is present (its path is the argument,
default /root/reference).  Two sources:
  1. the reference's Python model, src/01-python-serial/python_serial.py,
     imported as-is and run with numpy's global generator seeded;
  2. the reference's C serial and OpenMP models
     (src/02-C-serial/monte_carlo_serial.c, src/03-openMP/monte_carlo_omp.c),
     compiled unmodified from the reference tree against the oracle's GSL
     shim (oracle/Makefile target `ref`) and called through the reference
     plugin API.
Inputs are the seeded synthetic portfolios of riskgpu.synth, stored next to
the outputs so a change of generator is detected.
"""
import importlib.util
import io
import os
import sys
import contextlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "gpu-montecarlo-risk_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from riskgpu import synth  # noqa: E402
import mc_oracle  # noqa: E402


def load_python_reference(ref_root):
    path = os.path.join(ref_root, "src", "01-python-serial", "python_serial.py")
    spec = importlib.util.spec_from_file_location("python_serial", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main(ref_root="/root/reference"):
    mc_oracle.build(ref=True)
    ps = load_python_reference(ref_root)

    # 1. Python reference, on the 20-asset portfolio and on the module's own
    #    example parameters (python_serial.py:113-122, x=0.2 as written there).
    p = synth.one_factor_20()
    cases = {}
    np.random.seed(12345)
    with contextlib.redirect_stdout(io.StringIO()):
        P, count, S = ps.monte_carlo_crash_simulation(p.x, p.n, p.k, p.mu, p.sigma, 3000)
    cases["cfg20"] = dict(mu=p.mu, sigma=p.sigma, x=p.x, k=p.k, M=3000, seed=12345, P=P,
                          count=count, S=S.astype(np.int8))
    N = 10
    mu = np.zeros(N)
    Sigma = np.full((N, N), 0.3 * 0.04) + np.eye(N) * 0.04 * 0.7
    np.random.seed(7)
    with contextlib.redirect_stdout(io.StringIO()):
        P2, count2, S2 = ps.monte_carlo_crash_simulation(0.2, N, 5, mu, Sigma, 2000)
    cases["example10"] = dict(mu=mu, sigma=Sigma, x=0.2, k=5, M=2000, seed=7, P=P2, count=count2,
                              S=S2.astype(np.int8))
    out = {}
    for name, c in cases.items():
        for key, v in c.items():
            out[f"{name}__{key}"] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "python_serial.npz"), **out)

    # 2. Reference C models (serial: per-path S; OpenMP: counts), both
    #    upper-triangle semantics of the GSL factorisation.
    out = {"mu": p.mu, "sigma": p.sigma, "x": p.x, "k": p.k, "M": 5000, "seed": 42}
    with contextlib.redirect_stdout(io.StringIO()):
        for keep in (1, 0):
            r, S = mc_oracle.ref_run("serial", p.mu, p.sigma, 5000, p.k, p.x, 42, keep, True)
            out[f"serial_keep{keep}_S"] = S.astype(np.int8)
            out[f"serial_keep{keep}_count"] = r["count"]
            out[f"serial_keep{keep}_stats"] = np.array([r["P_hat"], r["std_error"], r["ci_lower"], r["ci_upper"]])
            ro = mc_oracle.ref_run("openmp", p.mu, p.sigma, 5000, p.k, p.x, 42, keep)
            out[f"openmp_keep{keep}_count"] = ro["count"]
    np.savez_compressed(os.path.join(HERE, "ref_c_serial.npz"), **out)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main(*sys.argv[1:])

"""C ABI checks that need no GPU: the library builds and loads, exports every
symbol the public headers declare, and rejects invalid requests before it
touches a device."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADERS = [os.path.join(ROOT, "include", h) for h in ("riskgpu.h", "riskgpu_plugin.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        src = re.sub(r"^\s*typedef[^;]*;", "", src, flags=re.M)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", src, re.M):
            name = m.group(1)
            if name not in ("if", "while", "for", "return", "sizeof"):
                names.add(name)
    names.discard("ModelRunFunc")
    return names


def test_headers_compile_as_c(engine, tmp_path):
    c = tmp_path / "h.c"
    c.write_text('#include "riskgpu.h"\n#include "riskgpu_plugin.h"\nint main(void){return 0;}\n')
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "gpu-montecarlo-risk_gb300", "csrc", "gslabi"), "-c", str(c),
                    "-o", str(tmp_path / "h.o")], check=True)


def test_exports_every_declared_symbol(engine):
    decl = declared_functions()
    assert decl == set(engine.EXPORTED_SYMBOLS), decl ^ set(engine.EXPORTED_SYMBOLS)
    out = subprocess.run(["nm", "-D", "--defined-only", engine.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    missing = decl - exported
    assert not missing, missing


def test_plugin_struct_layout_matches_reference_header(engine, tmp_path):
    """sizeof/offsetof of the plugin structures equal those of the reference's
    own src/model_interface.h (compiled here when the reference tree exists)
    and of the ctypes mirror."""
    prog = r'''
#include <stdio.h>
#include <stddef.h>
#include HEADER
int main(void){
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(MonteCarloParams), sizeof(MonteCarloResult),
    offsetof(MonteCarloParams, mu), offsetof(MonteCarloParams, M), offsetof(MonteCarloParams, random_seed),
    offsetof(MonteCarloResult, S_values), offsetof(MonteCarloResult, ci_upper), sizeof(ModelFunctions));
  return 0; }
'''
    inc = ["-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "gpu-montecarlo-risk_gb300", "csrc", "gslabi")]
    outs = []
    headers = ['"riskgpu_plugin.h"']
    if os.path.exists("/root/reference/src/model_interface.h"):
        headers.append('"/root/reference/src/model_interface.h"')
    for h in headers:
        c = tmp_path / "l.c"
        c.write_text(prog.replace("HEADER", h))
        exe = tmp_path / "l"
        subprocess.run(["gcc", "-std=gnu11"] + inc + [str(c), "-o", str(exe)], check=True)
        outs.append(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)
    assert len(set(outs)) == 1, outs
    r = engine
    vals = [int(v) for v in outs[0].split()]
    assert vals[0] == ctypes.sizeof(r.MonteCarloParams)
    assert vals[1] == ctypes.sizeof(r.MonteCarloResult)
    assert vals[2] == r.MonteCarloParams.mu.offset
    assert vals[3] == r.MonteCarloParams.M.offset
    assert vals[5] == r.MonteCarloResult.S_values.offset


def test_estimator_stats_and_tail_count(engine, oracle):
    p, se, lo, hi = engine.estimator_stats(4001326, 100_000_000)
    o = oracle.stats(4001326, 100_000_000)
    assert (p, se, lo, hi) == (o["P_hat"], o["std_error"], o["ci_lower"], o["ci_upper"])
    # published serial row of the reference (results/a.csv:3): 0.040013, SE 0.000020
    assert round(p, 6) == 0.040013 and round(se, 6) == 0.00002
    assert round(lo, 6) == 0.039975 and round(hi, 6) == 0.040052
    for M, a in [(1_000_000, 0.99), (100, 0.99), (150, 0.99), (1, 0.5), (12345, 0.975)]:
        assert engine.tail_count(M, a) == oracle.tail_count(M, a)


def test_invalid_requests_rejected_without_device(engine):
    """Validation happens before any device call, so these run on CPU."""
    L = engine.lib()
    h = ctypes.c_void_p()
    mu = np.zeros(3)
    sig = np.eye(3)
    assert L.rg_portfolio_create(0, mu.ctypes.data, sig.ctypes.data, 3, None, 0, ctypes.byref(h)) == engine.RG_ERR_INVALID
    assert L.rg_portfolio_create(3, None, sig.ctypes.data, 3, None, 0, ctypes.byref(h)) == engine.RG_ERR_INVALID
    assert L.rg_portfolio_create(3, mu.ctypes.data, sig.ctypes.data, 2, None, 0, ctypes.byref(h)) == engine.RG_ERR_INVALID
    bad = mu.copy(); bad[1] = np.nan
    assert L.rg_portfolio_create(3, bad.ctypes.data, sig.ctypes.data, 3, None, 0, ctypes.byref(h)) == engine.RG_ERR_INVALID
    badS = sig.copy(); badS[2, 1] = np.inf
    assert L.rg_portfolio_create(3, mu.ctypes.data, badS.ctypes.data, 3, None, 0, ctypes.byref(h)) == engine.RG_ERR_INVALID
    assert b"NaN or Inf" in L.rg_last_error()
    assert L.rg_portfolio_create(5000, mu.ctypes.data, sig.ctypes.data, 5000, None, 0, ctypes.byref(h)) == engine.RG_ERR_UNSUPPORTED
    # queries
    r = engine.Result()
    for q in (engine.make_query(0, 1), engine.make_query(10, 1, horizon=0),
              engine.make_query(10, 1, x=float("nan")), engine.make_query(10, 1, rng=7),
              engine.make_query(10, 1, var_level=1.0)):
        assert L.rg_run(3, mu.ctypes.data, sig.ctypes.data, 3, None, ctypes.byref(q), ctypes.byref(r)) == engine.RG_ERR_INVALID


def test_no_device_reported_cleanly(engine):
    if engine.lib().rg_device_count() > 0:
        pytest.skip("a device is present")
    r = engine.Result()
    q = engine.make_query(10, 1)
    mu = np.zeros(3); sig = np.eye(3)
    assert engine.lib().rg_run(3, mu.ctypes.data, sig.ctypes.data, 3, None, ctypes.byref(q), ctypes.byref(r)) == engine.RG_ERR_NO_DEVICE


def test_plugin_rejects_bad_params_without_device(engine):
    call = engine.PluginCall(np.zeros(4), np.eye(4))
    assert call.run(0, 2, 0.02, 1)["status"] == -1     # M = 0
    assert engine.lib().get_cuda_model().name == b"cuda"


def test_status_strings(engine):
    L = engine.lib()
    for s in range(0, -10, -1):
        assert L.rg_status_string(s) != b"unknown status"
    assert L.rg_abi_version() == 1

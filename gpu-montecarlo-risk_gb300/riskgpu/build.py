"""Build the engine in-tree: libriskgpu.so (sm_103a) and the C host runner.

Every CUDA translation unit is compiled for sm_103a only
(`-gencode arch=compute_103a,code=sm_103a`) in parallel, then linked into
one shared library with the C ABI of include/riskgpu.h and
include/riskgpu_plugin.h.  The runner is plain C linked against it.
A content hash of the sources skips work when nothing changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(PKG))
CSRC = os.path.join(os.path.dirname(PKG), "csrc")
RUNNER_DIR = os.path.join(os.path.dirname(PKG), "runner")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libriskgpu.so")
RUNNER = os.path.join(OUT, "riskgpu_runner")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-Wall", "-I" + INCLUDE,
           "-I" + os.path.join(CSRC, "gslabi")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine cannot be built")


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    deps = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
                  + glob.glob(os.path.join(CSRC, "gslabi", "**", "*"), recursive=True)
                  + glob.glob(os.path.join(RUNNER_DIR, "*.c")))
    return cu, deps


def _digest(files, extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for f in files:
        if os.path.isfile(f):
            h.update(f.encode())
            with open(f, "rb") as fh:
                h.update(fh.read())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the engine; returns the path of libriskgpu.so."""
    os.makedirs(OUT, exist_ok=True)
    cu, deps = _sources()
    nvcc = _nvcc()
    import platform
    digest = _digest(cu + deps, " ".join(ARCH + NVFLAGS) + platform.machine())
    stamp = os.path.join(OUT, "build.stamp")
    if (not force and os.path.exists(LIB) and os.path.exists(RUNNER) and os.path.exists(stamp)
            and open(stamp).read() == digest):
        return LIB
    objs = [os.path.join(OUT, os.path.basename(c)[:-3] + ".o") for c in cu]

    def compile_one(src_obj):
        src, obj = src_obj
        cmd = [nvcc] + ARCH + NVFLAGS + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(2, min(len(cu), os.cpu_count() or 4))) as ex:
        list(ex.map(compile_one, zip(cu, objs)))
    tmp = LIB + ".tmp"
    subprocess.run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs, check=True)
    os.replace(tmp, LIB)
    # C host runner (drop-in driver), linked against the engine.
    runner_src = [os.path.join(RUNNER_DIR, "riskgpu_runner.c"),
                  os.path.join(CSRC, "gslabi", "gsl_containers.c")]
    if all(os.path.exists(s) for s in runner_src):
        subprocess.run(["gcc", "-O2", "-std=gnu11", "-Wall", "-I" + INCLUDE,
                        "-I" + os.path.join(CSRC, "gslabi"), "-o", RUNNER] + runner_src +
                       ["-L" + OUT, "-lriskgpu", "-Wl,-rpath,$ORIGIN", "-lm"], check=True)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))

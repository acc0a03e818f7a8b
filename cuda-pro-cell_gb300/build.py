"""Build recipe for libprocell.so and the `procell` CLI (sm_103a only).

    python cuda-pro-cell_gb300/build.py          # or __graft_entry__.build()

Outputs go to cuda-pro-cell_gb300/build/ (git-ignored). Translation units compile in
parallel; the device code is built with --fmad=false and the host code with
-ffp-contract=off because the random stream's FP32/FP64 arithmetic must round
identically on the host and the device.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, out: str | None = None, defines=()) -> str:
    """Compile into `out` (default cuda-pro-cell_gb300/build). `defines` are extra
    -DNAME=VALUE macros for the device code (tuning variants)."""
    OUT = out or globals()["OUT"]
    os.makedirs(OUT, exist_ok=True)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    headers = [os.path.join(CSRC, h) for h in ("pc_rng.h", "pc_engine.h", "pc_sweeps.cuh", "pc_guard.h")] + \
        [os.path.join(INCLUDE, "procell.h")]
    host_flags = ["-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-fno-fast-math", "-Wall",
                  "-I" + os.path.join(cuda, "include"), "-I" + INCLUDE]
    jobs = []
    objs = []
    dflags = ["-D" + d for d in defines]
    for name in ("pc_kernels.cu", "pc_tuned_plain.cu", "pc_tuned_batched.cu", "pc_noalloc.cu", "pc_smooth.cu"):
        k_src = os.path.join(CSRC, name)
        k_obj = os.path.join(OUT, name.replace(".cu", ".o"))
        objs.append(k_obj)
        if defines or _stale(k_obj, [k_src] + headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xptxas", "-v",
                         "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + INCLUDE, *dflags, "-c", k_src,
                         "-o", k_obj])
    for name in ("pc_api.cpp", "pc_io.cpp"):
        src = os.path.join(CSRC, name)
        obj = os.path.join(OUT, name.replace(".cpp", ".o"))
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["g++", *host_flags, "-c", src, "-o", obj])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    lib = os.path.join(OUT, "libprocell.so")
    if defines or _stale(lib, objs):
        logs.append(_run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", lib, *objs, "-lpthread"]))
    cli_src = os.path.join(CSRC, "procell_cli.cpp")
    cli = os.path.join(OUT, "procell")
    if _stale(cli, [cli_src, lib, os.path.join(INCLUDE, "procell.h")]):
        logs.append(_run(["g++", "-O2", "-std=c++17", "-Wall", "-I" + INCLUDE, cli_src, "-o", cli,
                          "-L" + OUT, "-lprocell", "-Wl,-rpath,$ORIGIN"]))
    if verbose:
        sys.stdout.write("".join(logs))
    return lib


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None)
    ap.add_argument("--define", action="append", default=[])
    ap.add_argument("--quiet", action="store_true")
    a = ap.parse_args()
    print(build(verbose=not a.quiet, out=a.out, defines=a.define))

"""Build libflctgpu.so (the C-ABI library) in-tree with nvcc for sm_103a.

    python -m pyflct_gb300.build [--force] [--jobs N]

Every .cu under csrc/ is compiled to an object in parallel
(-gencode arch=compute_103a,code=sm_103a), then linked into
pyflct_gb300/libflctgpu.so with the static CUDA runtime.  Objects go to
pyflct_gb300/_build/ (git-ignored); a source is recompiled only when it or a
header changed.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libflctgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-std=c++20", "-O3", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-fvisibility=hidden", "-I", CSRC, "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libflctgpu.so")


def _stale(obj: str, src: str, headers: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers)


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) +
                     glob.glob(os.path.join(ROOT, "include", "*.h")))
    cc = nvcc()
    todo = []
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(o, s, headers):
            todo.append((s, o))

    # extra nvcc flags, e.g. -DFLCT_TC_PROFILE for the tensor-core kernel's
    # per-stage clock counters (objects then rebuild: pass --force)
    extra = os.environ.get("FLCT_NVCC_EXTRA", "").split()

    def run(so):
        s, o = so
        cmd = [cc] + ARCH + NVFLAGS + extra + ["-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(s)}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr)
        return s

    if todo:
        jobs = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(jobs) as ex:
            for s in ex.map(run, todo):
                if verbose:
                    print("compiled", os.path.basename(s))
    # relink when any object is newer than the library (also after a failed link)
    stale_lib = not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs)
    if todo or force or stale_lib:
        tmp = LIB + ".tmp"
        cmd = [cc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr)
        os.replace(tmp, LIB)
    build_cli(verbose)
    build_probe(verbose)
    return LIB


PROBE_SRC = os.path.join(PKG, "probe", "fp32_peak.cu")
PROBE_LIB = os.path.join(PKG, "libflctprobe.so")


def build_probe(verbose: bool = False) -> str:
    """libflctprobe.so: the FP32-pipe throughput microbenchmark the bench
    uses as the FP32 form's roofline denominator (not part of the C ABI)."""
    if os.path.exists(PROBE_LIB) and os.path.getmtime(PROBE_LIB) >= os.path.getmtime(PROBE_SRC):
        return PROBE_LIB
    tmp = PROBE_LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-O3", "-Xcompiler", "-fPIC", "-shared", "-cudart", "static", PROBE_SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building the FP32 probe failed:\n" + r.stderr)
    if verbose and r.stderr.strip():
        print(r.stderr)
    os.replace(tmp, PROBE_LIB)
    return PROBE_LIB


CLI = os.path.join(PKG, "cli")
BIN = os.path.join(PKG, "bin")


def cc() -> str:
    for cand in (os.environ.get("CC"), shutil.which("gcc"), shutil.which("cc")):
        if cand and shutil.which(cand):
            return cand
    raise RuntimeError("a C compiler (gcc) is required to build the flct / warp programs")


def build_cli(verbose: bool = False) -> list[str]:
    """The `flct` and `warp` programs (C over the C ABI) in pyflct_gb300/bin,
    linked against libflctgpu.so with an rpath to it."""
    os.makedirs(BIN, exist_ok=True)
    out = []
    srcs = [os.path.join(CLI, "vcio.c")]
    deps = srcs + [os.path.join(CLI, "vcio.h"), os.path.join(ROOT, "include", "flct_gpu.h"), LIB]
    for prog in ("flct", "warp"):
        main_c = os.path.join(CLI, f"{prog}_main.c")
        exe = os.path.join(BIN, prog)
        out.append(exe)
        if os.path.exists(exe) and all(os.path.getmtime(exe) >= os.path.getmtime(d) for d in deps + [main_c]):
            continue
        cmd = [cc(), "-std=c11", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), main_c] + srcs + \
              ["-L", PKG, "-lflctgpu", "-Wl,-rpath,$ORIGIN/..", "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"building {prog} failed:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    print(build(a.force, a.jobs, a.verbose))


if __name__ == "__main__":
    sys.exit(main())

"""Builds libflutas_gb300.so in-tree with nvcc for sm_103a (no cmake, no torch).

Translation units are compiled in parallel, then linked with -shared.
Usage: python -m flutas_gb300.build   (or flutas_gb300.build.build()).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libflutas_gb300.so")
BUILD_DIR = os.path.join(HERE, "_build")

SOURCES = ["flutas_gb300.cu", "server.cu", "fixed.cu", "io.cu", "grid.cu", "mom.cu"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-Xcompiler", "-fvisibility=hidden"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build flutas_gb300")


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "flutas_gb300.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([cc, *ARCH, *NVFLAGS, "-c", s, "-o", o])
    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        run([cc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


EMU_LIB = os.path.join(HERE, "libflutas_emu.so")


def build_emu(verbose: bool = False) -> str:
    """Host-only build of the transform passes (CPU emulator used by the tests)."""
    src = os.path.join(CSRC, "emu.cu")
    deps = [src] + [os.path.join(CSRC, f) for f in ("fft_engine.cuh", "axis_tables.cuh", "fft_fixed.cuh", "bits.cuh",
                                                   "ghosts.cuh", "ptrcheck.h", "fft_ext.cuh", "dd.cuh")]
    if _stale(EMU_LIB, deps):
        cmd = [nvcc(), "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-shared",
               "--expt-relaxed-constexpr",
               "-o", EMU_LIB, src]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{r.stdout}\n{r.stderr}")
    return EMU_LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)

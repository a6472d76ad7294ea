"""Build recipe for libnbgb.so (the sm_103a CUDA library behind include/nbgb.h).

Every ``csrc/*.cu`` is compiled in parallel with nvcc for ``sm_103a`` only and
linked into ``nbgb/libnbgb.so`` inside the source tree (git-ignored).  A
rebuild happens when any source or header is newer than the library.
"""
from __future__ import annotations

import glob
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)  # nbody-gpu-sim_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD_DIR = os.path.join(ROOT, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libnbgb.so")
APP_SRC = os.path.join(ROOT, "app", "nbgb_sim.cpp")
APP_PATH = os.path.join(PKG_DIR, "nbgb_sim")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC] + ARCH


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def is_stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(p) > t for p in sources() + _headers() + [__file__])


def build_app(force: bool = False) -> str:
    """The headless driver ``nbgb_sim`` (host C++ over libnbgb.so, rpath to
    its own directory); FP contraction off so its initial conditions are
    evaluated like the reference's host code."""
    if (not force and os.path.exists(APP_PATH) and
            os.path.getmtime(APP_PATH) >= max(os.path.getmtime(APP_SRC), os.path.getmtime(LIB_PATH),
                                              os.path.getmtime(os.path.join(INCLUDE, "nbgb.h")))):
        return APP_PATH
    cxx = os.environ.get("CXX", "g++")
    tmp = APP_PATH + ".tmp"
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", "-I", INCLUDE, APP_SRC,
                        "-o", tmp, "-L", PKG_DIR, "-lnbgb", "-Wl,-rpath,$ORIGIN"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed for nbgb_sim:\n" + r.stdout + r.stderr)
    os.replace(tmp, APP_PATH)
    return APP_PATH


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    """Compile and link libnbgb.so (and the nbgb_sim driver); returns the
    library path."""
    if not force and not is_stale():
        build_app()
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    flags = NVCC_FLAGS + (extra_flags or [])
    jobs, objs = [], []
    hdr_t = max((os.path.getmtime(h) for h in _headers()), default=0.0)
    for src in sources():
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_t, os.path.getmtime(__file__)):
            jobs.append([nvcc] + flags + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=min(16, max(1, len(jobs)))) as ex:
        list(ex.map(_run, jobs))
    tmp = LIB_PATH + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs)
    os.replace(tmp, LIB_PATH)
    build_app(force=True)
    if verbose:
        print("built", LIB_PATH, "and", APP_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))

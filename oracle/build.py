"""Build recipe for the parity checker (test infrastructure only).

* ``oracle/liboracle.so``: the C restatement in ``nbody_oracle.c``, built with
  ``-ffp-contract=off`` (see that file's header) and OpenMP.
* ``oracle/_ref/libnbody_ref.so``: the reference's own host-side code,
  compiled in place from the reference sources plus ``ref_harness.cpp``.  Only
  built where NBGB_REFERENCE_ROOT names the reference tree; outputs go to
  ``oracle/_ref/`` only.

Usage: ``NBGB_REFERENCE_ROOT=<reference tree> python oracle/build.py [--ref]``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference tree is named by NBGB_REFERENCE_ROOT; a build of
# oracle/_ref records the tree it used (oracle/_ref/source_root), so later
# processes find it without the variable.  Without either, only an already
# built oracle/_ref library is used.
REF_ROOT = os.environ.get("NBGB_REFERENCE_ROOT", "")
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_DIR, "libnbody_ref.so")

# Reference sources whose host code the harness drives (relative to the
# reference root).  They are compiled where they lie; nothing is copied.
_REF_CU = ["src/cuda/force_direct.cu", "src/cuda/force_barnes_hut.cu",
           "src/cuda/force_spatial_hash.cu", "src/cuda/particle_init.cu"]
_REF_CPP = ["src/utils/error_handling.cpp", "src/utils/performance_observability.cpp",
            "src/utils/serialization.cpp", "src/utils/simulation_state.cpp"]
_REF_DEFS = ["-DNDEBUG", "-DNBODY_WITH_CUDA=1", "-DNBODY_WITH_RENDERING=0",
             "-DNBODY_WITH_UI=0", "-DNBODY_ENABLE_PROFILING=0"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "nbody_oracle.c")
    if force or _stale(LIB, [src]):
        tmp = LIB + ".tmp"
        _run(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-shared",
              "-fPIC", "-std=c11", src, "-o", tmp, "-lm"])
        os.replace(tmp, LIB)
    return LIB


def _ref_root() -> str:
    root = os.environ.get("NBGB_REFERENCE_ROOT", REF_ROOT)
    rec = os.path.join(REF_DIR, "source_root")
    if not root and os.path.isfile(rec):
        with open(rec) as f:
            root = f.read().strip()
    return root


def reference_available() -> bool:
    root = _ref_root()
    return bool(root) and os.path.isfile(os.path.join(root, "src/cuda/force_barnes_hut.cu"))


def build_ref(force: bool = False) -> str | None:
    """Compile the reference host code + harness into oracle/_ref (CPU use only).
    Without the reference sources, an earlier build of the library is used."""
    if not reference_available():
        return REF_LIB if os.path.isfile(REF_LIB) else None
    root = _ref_root()
    harness = os.path.join(HERE, "ref_harness.cpp")
    srcs = [os.path.join(root, s) for s in _REF_CU + _REF_CPP] + [harness]
    if not (force or _stale(REF_LIB, srcs)):
        return REF_LIB
    os.makedirs(REF_DIR, exist_ok=True)
    inc = ["-I", os.path.join(root, "include")]
    # The reference is built with separable compilation (its CMakeLists sets
    # CUDA_SEPARABLE_COMPILATION); the kernels are compiled but never run here.
    nv = ["nvcc", "-std=c++17", "-O3", "-rdc=true", "-Xcompiler", "-fPIC",
          "-gencode", "arch=compute_103a,code=sm_103a"] + _REF_DEFS + inc
    gx = ["g++", "-std=c++17", "-O3", "-fPIC", "-I", "/usr/local/cuda/include"] + _REF_DEFS + inc
    jobs, objs = [], []
    for s in _REF_CU:
        o = os.path.join(REF_DIR, os.path.basename(s) + ".o")
        jobs.append(nv + ["-c", os.path.join(root, s), "-o", o])
        objs.append(o)
    for s in _REF_CPP:
        o = os.path.join(REF_DIR, os.path.basename(s) + ".o")
        jobs.append(gx + ["-c", os.path.join(root, s), "-o", o])
        objs.append(o)
    ho = os.path.join(REF_DIR, "ref_harness.o")
    jobs.append(gx + ["-c", harness, "-o", ho])
    objs.append(ho)
    with ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(_run, jobs))
    _run(["nvcc", "-shared", "-rdc=true", "-gencode", "arch=compute_103a,code=sm_103a",
          "-cudart", "shared", "-Xlinker", "-Bsymbolic", *objs, "-o", REF_LIB])
    with open(os.path.join(REF_DIR, "source_root"), "w") as f:
        f.write(root + "\n")
    return REF_LIB


def link_reference_apps(lib_dir: str) -> dict[str, str] | None:
    """Link check of the drop-in: the reference's unchanged benchmark driver,
    ParticleSystem, utilities and one example, with the hot-path classes
    supplied by nbody-gpu-sim_gb300/adapter/nbody_adapter.cpp and the
    kernels by libnbgb.so in lib_dir.  Outputs go to oracle/_ref/link/.
    Returns {app: path} or None where the reference sources are absent."""
    if not reference_available():
        return None
    root = _ref_root()
    repo = os.path.dirname(HERE)
    out = os.path.join(REF_DIR, "link")
    os.makedirs(out, exist_ok=True)
    inc = ["-I", os.path.join(root, "include"), "-I", os.path.join(repo, "include"),
           "-I", "/usr/local/cuda/include"]
    defs = ["-DNDEBUG", "-DNBODY_WITH_CUDA=1", "-DNBODY_WITH_RENDERING=0", "-DNBODY_WITH_UI=0",
            "-DNBODY_ENABLE_PROFILING=1"]
    srcs = ["src/core/particle_system.cpp", "src/utils/error_handling.cpp",
            "src/utils/performance_observability.cpp", "src/utils/serialization.cpp",
            "src/utils/simulation_state.cpp"]
    jobs, objs = [], []
    for s in srcs:
        o = os.path.join(out, os.path.basename(s) + ".o")
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC"] + defs + inc +
                    ["-c", os.path.join(root, s), "-o", o])
        objs.append(o)
    # particle_init.cu holds host code only (allocation, copies, initialisers)
    o = os.path.join(out, "particle_init.cu.o")
    jobs.append(["nvcc", "-std=c++17", "-O2", "-Xcompiler", "-fPIC",
                 "-gencode", "arch=compute_103a,code=sm_103a"] + defs + inc +
                ["-c", os.path.join(root, "src/cuda/particle_init.cu"), "-o", o])
    objs.append(o)
    ad = os.path.join(out, "nbody_adapter.o")
    jobs.append(["g++", "-std=c++17", "-O2", "-fPIC"] + defs + inc +
                ["-c", os.path.join(repo, "nbody-gpu-sim_gb300", "adapter", "nbody_adapter.cpp"),
                 "-o", ad])
    objs.append(ad)
    mains = {"nbody_benchmarks": "benchmarks/benchmark_main.cpp",
             "example_basic": "examples/example_basic.cpp"}
    for app, s in mains.items():
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC"] + defs + inc +
                    ["-c", os.path.join(root, s), "-o", os.path.join(out, app + ".o")])
    with ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(_run, jobs))
    apps = {}
    for app in mains:
        exe = os.path.join(out, app)
        _run(["g++", "-o", exe, os.path.join(out, app + ".o")] + objs +
             ["-L", lib_dir, "-lnbgb", "-Wl,-rpath," + lib_dir, "-L", "/usr/local/cuda/lib64",
              "-lcudart", "-lpthread"])
        apps[app] = exe
    return apps


def link_adapter_runtime() -> str | None:
    """The drop-in adapter (nbody-gpu-sim_gb300/adapter/nbody_adapter.cpp)
    with the reference's error-handling and profiling sources, linked
    against the fake C ABI of tests/adapter_runtime/fake_nbgb.c and driven
    by tests/adapter_runtime/driver.cpp: a CPU check of the adapter's own
    logic.  Outputs go to oracle/_ref/link/.  Returns the driver's path, or
    None where the reference sources are absent."""
    if not reference_available():
        return None
    root = _ref_root()
    repo = os.path.dirname(HERE)
    src = os.path.join(repo, "tests", "adapter_runtime")
    out = os.path.join(REF_DIR, "link")
    os.makedirs(out, exist_ok=True)
    fake = os.path.join(out, "libnbgb_fake.so")
    _run(["gcc", "-std=c11", "-O1", "-fPIC", "-shared", "-I", os.path.join(repo, "include"),
          os.path.join(src, "fake_nbgb.c"), "-o", fake])
    inc = ["-I", os.path.join(root, "include"), "-I", os.path.join(repo, "include"),
           "-I", "/usr/local/cuda/include"]
    defs = ["-DNDEBUG", "-DNBODY_WITH_CUDA=1", "-DNBODY_WITH_RENDERING=0", "-DNBODY_WITH_UI=0",
            "-DNBODY_ENABLE_PROFILING=1"]
    srcs = [os.path.join(repo, "nbody-gpu-sim_gb300", "adapter", "nbody_adapter.cpp"),
            os.path.join(src, "driver.cpp"),
            os.path.join(root, "src/utils/error_handling.cpp"),
            os.path.join(root, "src/utils/performance_observability.cpp")]
    exe = os.path.join(out, "adapter_runtime")
    _run(["g++", "-std=c++17", "-O1"] + defs + inc + srcs +
         ["-o", exe, "-L", out, "-lnbgb_fake", "-Wl,-rpath," + out,
          "-L", "/usr/local/cuda/lib64", "-lcudart", "-lpthread"])
    return exe


if __name__ == "__main__":
    print(build_oracle(force=True))
    if "--ref" in sys.argv:
        print(build_ref(force=True))

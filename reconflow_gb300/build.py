"""Build the in-tree CUDA library ``reconflow_gb300/lib/librfgb300.so``.

Every translation unit is compiled for sm_103a only, in parallel, with
``-fmad=false`` for the solver kernels (IEEE division / square root and no
multiply-add contraction, so results are a deterministic function of the
inputs) and linked into one shared library with the C ABI of
``include/reconflow_gb300.h``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "librfgb300.so")
OBJ_DIR = os.path.join(HERE, "_build")
# debug variant: every field access of the inner iteration checked against its
# plane (-DRF_BOUNDS_CHECK); out-of-range indices are counted, not followed
CHECK_LIB_PATH = os.path.join(LIB_DIR, "librfgb300_check.so")
CHECK_OBJ_DIR = os.path.join(HERE, "_build_check")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# per-file flags: the solver keeps exact IEEE arithmetic without contraction
SOURCES = {
    "rf_kernels.cu": ["-fmad=false"],
    "rf_solver.cu": ["-fmad=false"],
    "rf_noalloc.cu": ["-fmad=false"],
    "rf_batch.cu": ["-fmad=false"],
    # warm-start features and state (around the network, not on the parity path)
    "rf_warm.cu": [],
    # the learned warm start: BF16 tensor-core convolutions, FP32 accumulation
    "rf_cnn.cu": [],
    # pose front end: feature detection, description and matching (exact FP32,
    # compared bit for bit with the oracle) and the host-side relative pose
    "rf_pose.cu": ["-fmad=false"],
    "rf_epipolar.cpp": [],
}
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
          "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build reconflow_gb300")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    out = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    out += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return out


def build(force: bool = False, verbose: bool = False, bounds_check: bool = False) -> str:
    """Compile the library (only stale objects unless ``force``); with
    ``bounds_check`` the debug variant ``lib/librfgb300_check.so`` instead."""
    lib_path = CHECK_LIB_PATH if bounds_check else LIB_PATH
    obj_dir = CHECK_OBJ_DIR if bounds_check else OBJ_DIR
    extra = ["-DRF_BOUNDS_CHECK"] if bounds_check else []
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(obj_dir, exist_ok=True)
    nv = nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for src, flags in SOURCES.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(obj_dir, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nv, "-c", s, "-o", o] + ARCH + COMMON + extra + flags)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stdout + r.stderr

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for log in ex.map(run, jobs):
            if verbose and log.strip():
                print(log)
    if force or jobs or _stale(lib_path, objs):
        run([nv, "-shared", "-o", lib_path] + objs + ARCH + ["-Xcompiler", "-fPIC,-pthread",
                                                              "-lcudart_static", "-ldl", "-lrt",
                                                              "-lpthread"])
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                bounds_check="--bounds-check" in sys.argv))

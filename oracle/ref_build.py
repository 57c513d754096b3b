"""Compile the reference's own texture-free hot-path kernels for sm_103a.

Test infrastructure only: nothing in ``reconflow_gb300/`` or in a timed
region of ``bench.py`` loads what this makes.  The outputs pin the oracle to
the reference itself: ``tests/test_gpu_ref_pin.py`` launches each reference
kernel on the GPU and compares it bit for bit with the oracle's FP32 step.

The eight files below include only the reference's class headers
(``ReconFlow.h`` / ``CudaFlow.h``); those headers pull in OpenCV and the CUDA
Samples' ``helper_cuda.h``, which are absent, so this script writes a stub
class header into ``oracle/_ref/include/`` that declares exactly the member
functions the eight files define (their signatures are read from the files
themselves) plus the two block-size members and ``iDivUp`` that the launch
wrappers use.  The reference sources are compiled where they lie; nothing is
copied into the repository.  Outputs, all under ``oracle/_ref/``:

* ``ref_kernels_fmad0.fatbin``: built with ``-fmad=false`` (IEEE, no
  multiply-add contraction; the oracle's FP32 arithmetic).
* ``ref_kernels_fmad1.fatbin``: built with nvcc's default ``-fmad=true``, as
  the reference's Visual Studio project builds it (``reconflow.vcxproj`` sets
  no ``fmad`` option).
* ``kernels.json``: each ``__global__`` function's name, parameter types and
  Itanium-mangled symbol (for ``cuModuleGetFunction``).

The fatbins are device code only, so they load on any host through the CUDA
driver API (``oracle/ref_kernels.py``).  Run: ``python oracle/ref_build.py``
(``RF_REFERENCE_DIR`` overrides the reference checkout's location).
"""
from __future__ import annotations

import json
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF = os.environ.get("RF_REFERENCE_DIR", "/root/reference")
SRC = os.path.join(REF, "reconflow")

# the hot-path kernel files that use no texture references
FILES = ["solveReconDataL1.cu", "solveSmoothDualTVGlobal.cu", "solveUVProj.cu",
         "solve3dMinimalArea.cu", "solveUcSk.cu", "medianFilter.cu", "addKernel.cu",
         "solveDataL1.cu"]

_KERNEL = re.compile(r"__global__\s+void\s+(\w+)\s*\(([^)]*)\)", re.S)
_MEMBER = re.compile(r"^(void|int)\s+(ReconFlow|CudaFlow)\s*::\s*(\w+)\s*\(([^)]*)\)\s*\{",
                     re.S | re.M)
_COMMENT = re.compile(r"//[^\n]*|/\*.*?\*/", re.S)


def _strip_comments(text: str) -> str:
    return _COMMENT.sub(" ", text)


def param_type(decl: str) -> str:
    """'const float *u0' -> 'const float*'; 'int width' -> 'int'."""
    d = " ".join(decl.replace("*", " * ").split())
    toks = d.split(" ")
    if toks and toks[-1] not in ("*", "float", "int", "double", "const"):
        toks = toks[:-1]  # drop the parameter name
    out = " ".join(t for t in toks if t != "*") + "*" * toks.count("*")
    return out


# --- Itanium C++ ABI mangling of a free function with builtin / pointer / const params ---

_BUILTIN = {"float": "f", "int": "i", "double": "d", "void": "v", "char": "c",
            "unsigned int": "j", "bool": "b"}


def _type_tree(t: str):
    t = t.strip()
    if t.endswith("*"):
        return ("P", _type_tree(t[:-1]))
    if t.startswith("const "):
        return ("K", _type_tree(t[len("const "):]))
    return ("B", _BUILTIN[t])


def _seq_id(n: int) -> str:
    if n == 0:
        return ""
    n -= 1
    digits = "0123456789ABCDEFGHIJKLMNOPQRSTUVWXYZ"
    s = ""
    while True:
        s = digits[n % 36] + s
        n //= 36
        if n == 0:
            return s


def mangle(name: str, params) -> str:
    """Mangled symbol of ``void name(params...)`` at namespace scope."""
    subs: dict = {}

    def m(node):
        if node[0] == "B":
            return node[1]
        if node in subs:
            return "S" + _seq_id(subs[node]) + "_"
        s = node[0] + m(node[1])
        subs[node] = len(subs)
        return s

    body = "".join(m(_type_tree(p)) for p in params) if params else "v"
    return f"_Z{len(name)}{name}{body}"


def scan():
    """Kernels and class members defined in the reference files."""
    kernels, members = [], {"CudaFlow": [], "ReconFlow": []}
    for f in FILES:
        text = _strip_comments(open(os.path.join(SRC, f)).read())
        for name, plist in _KERNEL.findall(text):
            params = [param_type(p) for p in plist.split(",") if p.strip()]
            kernels.append({"file": f, "name": name, "params": params,
                            "symbol": mangle(name, params)})
        for ret, cls, name, plist in _MEMBER.findall(text):
            decl = f"{ret} {name}({' '.join(plist.split())});"
            if decl not in members[cls]:
                members[cls].append(decl)
    return kernels, members


def write_stub(members) -> str:
    inc = os.path.join(OUT, "include")
    os.makedirs(inc, exist_ok=True)
    cuda = "\n".join("    " + d for d in members["CudaFlow"])
    recon = "\n".join("    " + d for d in members["ReconFlow"])
    stub = f"""// Generated by oracle/ref_build.py: a stand-in for the reference's class
// headers, declaring only what its texture-free kernel files define and use.
#pragma once
#include <cuda_runtime.h>
#include <cmath>
static inline int iDivUp(int a, int b) {{ return (a % b != 0) ? (a / b + 1) : (a / b); }}
class CudaFlow {{
public:
    int BlockWidth = 32, BlockHeight = 8;
{cuda}
}};
class ReconFlow : public CudaFlow {{
public:
{recon}
}};
"""
    for nm in ("CudaFlow.h", "ReconFlow.h"):
        with open(os.path.join(inc, nm), "w") as fh:
            fh.write(stub)
    tu = os.path.join(OUT, "ref_kernels.cu")
    with open(tu, "w") as fh:
        fh.write("// Generated by oracle/ref_build.py: the reference's kernel files, unchanged.\n")
        for f in FILES:
            fh.write(f'#include "{os.path.join(SRC, f)}"\n')
    return tu


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build(force: bool = False) -> bool:
    """Build the fatbins if the reference checkout is present; returns False
    (and builds nothing) when it is not."""
    if not all(os.path.exists(os.path.join(SRC, f)) for f in FILES):
        return False
    kernels, members = scan()
    tu = write_stub(members)
    outs = {0: os.path.join(OUT, "ref_kernels_fmad0.fatbin"),
            1: os.path.join(OUT, "ref_kernels_fmad1.fatbin")}
    srcs = [os.path.join(SRC, f) for f in FILES] + [__file__]
    for fmad, path in outs.items():
        if not force and os.path.exists(path) and all(
                os.path.getmtime(path) >= os.path.getmtime(s) for s in srcs):
            continue
        cmd = [nvcc(), "-fatbin", tu, "-o", path, "-gencode", "arch=compute_103a,code=sm_103a",
               "-O3", "-std=c++17", f"-fmad={'true' if fmad else 'false'}",
               "-I" + os.path.join(OUT, "include"), "-w"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference kernels failed to build:\n{' '.join(cmd)}\n"
                               f"{r.stdout}\n{r.stderr}")
    with open(os.path.join(OUT, "kernels.json"), "w") as fh:
        json.dump({"files": FILES, "kernels": kernels,
                   "fatbins": {"fmad0": os.path.basename(outs[0]),
                               "fmad1": os.path.basename(outs[1])}}, fh, indent=1)
    return True


if __name__ == "__main__":
    ok = build(force="--force" in sys.argv)
    print("built" if ok else f"reference checkout not found at {SRC}: nothing built")

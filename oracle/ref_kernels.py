"""Launch the reference's own kernels (built by ``oracle/ref_build.py``).

Test infrastructure only: ``tests/test_gpu_ref_pin.py`` uses it to run the
reference kernels on the GPU beside the oracle; the library never loads it.
The fatbins hold device code only, so they are loaded through the CUDA
driver API (``libcuda.so.1`` via ctypes) into the context that PyTorch made
current, and each kernel is found by its mangled symbol from
``oracle/_ref/kernels.json``.
"""
from __future__ import annotations

import ctypes
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
MANIFEST = os.path.join(REF_DIR, "kernels.json")


def available(variant: str = "fmad0") -> bool:
    if not os.path.exists(MANIFEST):
        return False
    m = json.load(open(MANIFEST))
    return os.path.exists(os.path.join(REF_DIR, m["fatbins"][variant]))


class _Driver:
    def __init__(self):
        self.lib = ctypes.CDLL("libcuda.so.1")
        L = self.lib
        L.cuInit.argtypes = [ctypes.c_uint]
        L.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        L.cuModuleUnload.argtypes = [ctypes.c_void_p]
        L.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p,
                                          ctypes.c_char_p]
        L.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 6 + [
            ctypes.c_uint, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        L.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        self.check(L.cuInit(0), "cuInit")

    def check(self, rc, what):
        if rc != 0:
            s = ctypes.c_char_p()
            self.lib.cuGetErrorString(rc, ctypes.byref(s))
            raise RuntimeError(f"{what}: CUDA driver error {rc} "
                               f"({s.value.decode() if s.value else '?'})")


class RefKernels:
    """One loaded fatbin variant ("fmad0" or "fmad1")."""

    def __init__(self, variant: str = "fmad0"):
        import torch

        torch.cuda.init()
        torch.zeros(1, device="cuda")  # makes the primary context current on this thread
        self.torch = torch
        self.drv = _Driver()
        m = json.load(open(MANIFEST))
        self.kernels = {}
        for k in m["kernels"]:
            self.kernels.setdefault(k["name"], []).append(k)
        path = os.path.join(REF_DIR, m["fatbins"][variant]).encode()
        self.mod = ctypes.c_void_p()
        self.drv.check(self.drv.lib.cuModuleLoad(ctypes.byref(self.mod), path), "cuModuleLoad")
        self._fn = {}

    def close(self):
        if self.mod:
            self.drv.lib.cuModuleUnload(self.mod)
            self.mod = ctypes.c_void_p()

    def _function(self, name: str, n_params: int):
        cands = [k for k in self.kernels[name] if len(k["params"]) == n_params]
        if len(cands) != 1:
            raise KeyError(f"{name} with {n_params} parameters: {len(cands)} candidates")
        k = cands[0]
        if k["symbol"] not in self._fn:
            f = ctypes.c_void_p()
            self.drv.check(self.drv.lib.cuModuleGetFunction(ctypes.byref(f), self.mod,
                                                            k["symbol"].encode()),
                           f"cuModuleGetFunction({name})")
            self._fn[k["symbol"]] = (f, k["params"])
        return self._fn[k["symbol"]]

    def launch(self, name: str, grid, block, *args):
        """Launch ``name`` (overload chosen by argument count) on PyTorch's
        current stream.  Tensor arguments pass their device address; the
        parameter types from the manifest decide how scalars are passed."""
        f, types = self._function(name, len(args))
        holders = []
        for a, t in zip(args, types):
            if t.endswith("*"):
                holders.append(ctypes.c_void_p(0 if a is None else a.data_ptr()))
            elif t == "int":
                holders.append(ctypes.c_int(int(a)))
            elif t == "float":
                holders.append(ctypes.c_float(float(a)))
            else:
                raise TypeError(f"{name}: parameter type {t} not supported")
        params = (ctypes.c_void_p * len(holders))(
            *[ctypes.cast(ctypes.pointer(h), ctypes.c_void_p) for h in holders])
        gx, gy = grid
        bx, by = block
        stream = self.torch.cuda.current_stream().cuda_stream
        self.drv.check(self.drv.lib.cuLaunchKernel(f, gx, gy, 1, bx, by, 1, 0, stream, params,
                                                   None), f"cuLaunchKernel({name})")

    def launch2d(self, name: str, w: int, h: int, *args, block=(32, 8)):
        """The reference's launch shape: one thread per pixel of a w x h level."""
        bx, by = block
        self.launch(name, ((w + bx - 1) // bx, (h + by - 1) // by), block, *args)

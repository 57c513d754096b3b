"""The allocation-free per-warp update (rfk_warp_update_noalloc) for callers
that cannot allocate device memory where this step runs (a real-time pipeline
that forbids cudaMalloc after start-up, or a host framework that owns the
device memory budget).

It keeps its scratch planes in a static device array instead of taking them
from the caller; its results must equal rfk_warp_update's (the same kernels
with caller scratch) bit for bit, on consecutive calls that reuse the array.
This file is collected last so a run that stops at the first failure has run
everything else first; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from helpers import assert_bitexact

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _P(t):
    return ctypes.c_void_p(t.data_ptr())


def _inputs(torch, rng, w, h, s):
    n = (h + 1) * s
    arrs = [rng.normal(size=n).astype(np.float32) for _ in range(2)]
    arrs += [(rng.normal(size=n) * 3).astype(np.float32) for _ in range(2)]
    return [torch.from_numpy(a).cuda() for a in arrs]


def test_noalloc_matches_caller_scratch_on_consecutive_calls(torch_cuda):
    from reconflow_gb300 import _native

    lib = _native.load()
    rng = np.random.default_rng(21)
    # two calls in a row (different sizes, so the second reuses the static
    # array after the first left other data in it), each against the
    # caller-scratch entry point
    for (w, h, s) in ((1280, 720, 1280), (37, 23, 64), (1920, 1088, 1920)):
        d = _inputs(torch_cuda, rng, w, h, s)
        tmp = [torch_cuda.zeros_like(d[0]) for _ in range(2)]
        ref = [torch_cuda.zeros_like(d[0]) for _ in range(2)]
        out = [torch_cuda.full_like(d[0], 7.0) for _ in range(2)]
        _native.check(lib.rfk_warp_update(*[_P(t) for t in d], w, h, s, *[_P(t) for t in tmp],
                                          *[_P(t) for t in ref], None))
        _native.check(lib.rfk_warp_update_noalloc(*[_P(t) for t in d], w, h, s,
                                                  *[_P(t) for t in out], None))
        torch_cuda.cuda.synchronize()
        for a, b, nm in zip(out, ref, "uv"):
            assert_bitexact(a.cpu().numpy().reshape(h + 1, s), b.cpu().numpy().reshape(h + 1, s),
                            f"{nm} {w}x{h}", region=(h, w))


def test_noalloc_rejects_frames_beyond_the_static_scratch(torch_cuda):
    from reconflow_gb300 import _native

    lib = _native.load()
    w, h, s = 2048, 1080, 2048  # 2 211 840 floats per plane > 2 097 152
    t = torch_cuda.zeros(8, dtype=torch_cuda.float32, device="cuda")
    st = lib.rfk_warp_update_noalloc(*[_P(t)] * 4, w, h, s, _P(t), _P(t), None)
    assert st == 1  # RF_ERR_INVALID_ARG
    msg = lib.rf_last_error_string().decode()
    assert "exceeds the static scratch plane" in msg

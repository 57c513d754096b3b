"""Host logic of bench.py that runs without a GPU: the order of the calls in
the end-to-end serving loop (pipelined transfers), against a batch stand-in
that records them."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _Batch:
    def __init__(self, log, name):
        self.log, self.name = log, name

    def stageUpload(self, a, b, pitch):
        self.log.append((self.name, "up", a, b, pitch))

    def takeUpload(self):
        self.log.append((self.name, "take"))

    def stageDownload(self, pitch, u=None, v=None, inv_depth=None, X=None, Y=None, Z=None):
        self.log.append((self.name, "down", u, v, inv_depth, X, Y, Z, pitch))

    def waitDownload(self):
        self.log.append((self.name, "wait"))


def test_serving_loop_moves_every_step_once_in_order(monkeypatch):
    torch = pytest.importorskip("torch")
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    bench = _bench()
    log = []
    cols = [[f"c{k}"] for k in range(8)]
    items = [(_Batch(log, "A"), cols, 64), (_Batch(log, "B"), cols, 32)]
    steps = 3

    def step():
        log.append(("step",))

    t = bench.serve_pipelined(items, step, steps)
    assert t >= 0.0
    names = [e[1] if e[0] != "step" else "step" for e in log]
    # batch 0's frames first, then per step: take, next upload (not after
    # the last step), the solve, the download; the waits at the end
    want = ["up", "up"]
    for k in range(steps):
        want += ["take", "up", "take", "up"] if k + 1 < steps else ["take", "take"]
        want += ["step", "down", "down"]
    want += ["wait", "wait"]
    assert names == want
    assert sum(1 for e in log if e[0] != "step" and e[1] == "up") == steps * 2
    assert sum(1 for e in log if e[0] != "step" and e[1] == "down") == steps * 2
    # each batch's own columns and pitch
    assert ("A", "up", ["c0"], ["c1"], 64) in log and ("B", "up", ["c0"], ["c1"], 32) in log
    assert ("A", "down", ["c2"], ["c3"], ["c4"], ["c5"], ["c6"], ["c7"], 64) in log

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


def test_learned_schedules_match_the_package():
    """The bench's learned workloads refine with the schedules the package
    defines (reconflow_gb300.warmstart.SCHEDULES), which the fallback
    calibration also uses."""
    import bench
    from reconflow_gb300.warmstart import SCHEDULES

    wl = bench.WORKLOADS["720p-learned"]
    assert SCHEDULES[(1280, 720)] == dict(warm_level=wl["warm_level"], warps=wl["warm_warps"],
                                          iters=wl["warm_iters"])
    for key in ("mixed-4k-1080p-learned", "c5-stream"):
        for g in bench.WORKLOADS[key]["groups"]:
            sch = SCHEDULES[(g["width"], g["height"])]
            assert sch == dict(warm_level=g["warm_level"], warps=g["warm_warps"],
                               iters=g["warm_iters"])
            if "temporal_iters" in g:
                assert g["temporal_iters"] == sch["iters"]
                assert g["temporal_warps"] == sch["warps"]


def test_fallback_ceiling_and_test(tmp_path):
    """The deployable fallback test: non-finite energies always fall back,
    finite ones above the table's per-pixel ceiling do; a size without an
    entry has no ceiling."""
    import json
    import math

    from reconflow_gb300 import fallback as FB

    table = {"margin": 0.02, "entries": {"1280x720/network": {"ceiling": 3.0}}}
    p = tmp_path / "t.json"
    p.write_text(json.dumps(table))
    t = FB.load(str(p))
    c = FB.ceiling(t, 1280, 720, "network")
    assert c == 3.0 and FB.ceiling(t, 640, 480, "network") is None
    npx = 1280 * 720
    assert not FB.over(2.9 * npx, npx, c)
    assert FB.over(3.1 * npx, npx, c)
    assert FB.over(math.nan, npx, c) and FB.over(math.inf, npx, None)
    assert not FB.over(1e9, npx, None)
    # the committed table covers the bench's sizes and sources
    committed = FB.load()
    for key in ("1280x720/network", "1920x1080/network", "3840x2160/network"):
        ent = committed["entries"][key]
        assert ent["ceiling"] > ent["energy_per_px_max"] > 0
    for key in ("1920x1080/temporal", "3840x2160/temporal"):
        ent = committed["entries"][key]
        assert ent["history_factor"] == FB.HISTORY_FACTOR and ent["pairs"] >= 64
        assert 0 < ent["history_ratio_median"] <= ent["history_ratio_max"]
        assert FB.ceiling(committed, *map(int, key.split("/")[0].split("x")), "temporal") is None


def test_sequence_guard():
    """Along a sequence a pair falls back when its energy per pixel exceeds
    twice the median of the sequence's last three; the first pair is held
    to the network ceiling; a single outlier does not move the median, a
    lasting change is accepted after two pairs; sequences are independent."""
    import math

    from reconflow_gb300 import fallback as FB

    g = FB.SequenceGuard(2)
    px = 100
    assert g.over(0, 5.0 * px, px, 4.0)          # first pair over the network ceiling
    g.reset()
    assert not g.over(0, 2.0 * px, px, 4.0)
    assert not g.over(1, 9.0 * px, px, None)     # no ceiling: the first pair passes
    seq = [2.2, 2.4, 2.6, 7.0, 2.8, 3.0]         # one outlier (7.0 > 2 x 2.4)
    flags = [g.over(0, e * px, px, 4.0) for e in seq]
    assert flags == [False, False, False, True, False, False]
    assert g.over(0, math.nan, px, 4.0) and len(g.hist[0]) == 3   # NaN kept out
    flags = [g.over(0, e * px, px, 4.0) for e in (8.0, 8.5, 9.0)]  # a lasting jump
    assert flags == [True, True, False]
    assert g.hist[1] == [9.0]


def test_iterations_per_launch_table_entry():
    """The single-pair table's iterations-per-launch choice reaches
    rf_set_cluster_pixels; a table without one leaves the library alone."""
    from reconflow_gb300 import autotune

    class Lib:
        got = []

        def rf_set_cluster_pixels(self, n):
            self.got.append(n)

    lib = Lib()
    autotune.apply_iterations_per_launch(lib, {"levels": []})
    assert lib.got == []
    autotune.apply_iterations_per_launch(lib, {"iterations_per_launch": {"cluster_px": 4000}})
    assert lib.got == [4000]
    assert autotune.CLUSTER_CANDIDATES[0] == 0  # one iteration per launch is always a candidate

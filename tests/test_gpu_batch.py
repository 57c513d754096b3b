"""Batched solve on the GPU: every pair of a mixed-size batch must be bit for
bit what the single-pair solver (and the FP32 oracle) gives for that pair
alone, whatever its neighbours in the batch."""
import numpy as np
import pytest

from helpers import align_up, assert_bitexact, pad_rows, textured_pair

pytestmark = pytest.mark.gpu

SIZES = [(37, 23), (64, 48), (96, 64), (45, 90), (130, 70)]


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _pose(seed):
    rng = np.random.default_rng(seed)
    a = rng.normal(size=3)
    a /= np.linalg.norm(a)
    ang = np.radians(rng.uniform(0.5, 2.0))
    Kx = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    R = np.eye(3) + np.sin(ang) * Kx + (1 - np.cos(ang)) * Kx @ Kx
    t = rng.normal(size=3)
    return R, 0.1 * t / np.linalg.norm(t)


def _K(w, h):
    f = 500.0 * w / 640.0
    return np.array([[f, 0, w / 2.0], [0, f, h / 2.0], [0, 0, 1.0]])


def _inputs():
    out = []
    for i, (w, h) in enumerate(SIZES):
        rng = np.random.default_rng(100 + i)
        I0, I1 = textured_pair(rng, h, w, shift=(1.2 + 0.1 * i, -0.5))
        R, t = _pose(i)
        out.append((w, h, I0, I1, _K(w, h), R, t))
    return out


@pytest.mark.parametrize("fix,pipeline", [(0, "0"), (1, "0"), (1, "1")])
def test_batch_recon_matches_single_pair(oracle, rf, fix, pipeline, monkeypatch):
    """pipeline "1": the two pair groups half an inner iteration apart
    (RF_BATCH_PIPELINE, read when the batch is created)."""
    monkeypatch.setenv("RF_BATCH_PIPELINE", pipeline)
    L, warps, iters = 2, 2, 4
    data = _inputs()
    kw = dict(lambda_=50.0, lambdaf=0.1, lambdams=100.0, alphaTv=1 / 0.33, alphaProj=60.0,
              tau=0.25, nWarpIters=warps, nSolverIters=iters, fix_quirks=fix)
    b = rf.ReconFlowBatch([(w, h) for w, h, *_ in data], L, method=14, **kw)
    for i, (w, h, I0, I1, K, R, t) in enumerate(data):
        s = b.strides[i]
        b.setCameraMatrices(i, K, K)
        b.copyImagesToDevice(i, pad_rows(I0, s), pad_rows(I1, s))
    b.solveR([d[5] for d in data], [d[6] for d in data])
    E = b.energies()  # one batched evaluation of every pair
    # the queued form into pinned memory gives the same values once the
    # batch's stream has reached them
    import ctypes

    lib = rf.load()
    pe = ctypes.c_void_p()
    rf._native.check(lib.rf_host_alloc(8 * b.n, ctypes.byref(pe)))
    try:
        b.energiesAsync(pe.value)
        b.synchronize()
        Ea = np.ctypeslib.as_array(ctypes.cast(pe, ctypes.POINTER(ctypes.c_double)),
                                   shape=(b.n,)).copy()
    finally:
        lib.rf_host_free(pe)
    assert Ea.tobytes() == np.asarray(E, np.float64).tobytes()
    for i, (w, h, I0, I1, K, R, t) in enumerate(data):
        s = align_up(w)
        got_u, got_v = b.copyOpticalFlowToHost(i)
        X, Y, Z = b.copy3dToHost(i)
        f = rf.ReconFlow()
        f.initializeR(w, h, 1, L, 2.0, 14, 50.0, 0.0, 0.1, 100.0, 1 / 0.33, 60.0, 0.5, 0.25, warps,
                      iters, cvType=5, fix_quirks=fix)
        f.setCameraMatrices(K, K)
        f.copyImagesToDevice(pad_rows(I0, s), pad_rows(I1, s))
        f.solveR(R, t, 5.0)
        u1, v1 = f.copyOpticalFlowToHost()
        X1, Y1, Z1 = f.copy3dToHost()
        for a, c, nm in ((got_u, u1, "u"), (got_v, v1, "v"), (X, X1, "X"), (Y, Y1, "Y"), (Z, Z1, "Z")):
            assert_bitexact(a, c, f"pair {i} {nm}", region=(h, w))
        e1 = f.energy()
        assert np.float64(E[i]).tobytes() == np.float64(e1).tobytes(), (i, E[i], e1)
        if i == 2:
            p = oracle.make_params(w, h, L, lam=50.0, lambdaf=0.1, lambdams=100.0,
                                   alpha_tv=1 / 0.33, alpha_proj=60.0, tau=0.25,
                                   n_warp_iters=warps, n_solver_iters=iters, fix_quirks=fix)
            ref = oracle.solve(p, pad_rows(I0, s), pad_rows(I1, s), K0=K, K1=K, R1=R, t1=t,
                               dtype=np.float32)
            assert_bitexact(got_u, ref["u"], "oracle u", region=(h, w))
            assert_bitexact(Z, ref["Z"], "oracle Z", region=(h, w))
        inv = b.copyInverseDepthToHost(i)
        with np.errstate(divide="ignore"):
            np.testing.assert_array_equal(inv[:, :w], np.float32(1) / Z[:, :w])


def test_batch_plain_matches_single_pair(rf):
    L, warps, iters = 2, 2, 5
    data = _inputs()
    b = rf.ReconFlowBatch([(w, h) for w, h, *_ in data], L, method=0, lambda_=50.0, theta=0.33,
                          tau=0.25, nWarpIters=warps, nSolverIters=iters)
    for i, (w, h, I0, I1, *_r) in enumerate(data):
        s = b.strides[i]
        b.copyImagesToDevice(i, pad_rows(I0, s), pad_rows(I1, s))
    b.solveOpticalFlow()
    for i, (w, h, I0, I1, *_r) in enumerate(data):
        s = align_up(w)
        u, v = b.copyOpticalFlowToHost(i)
        f = rf.CudaFlow()
        f.initialize(w, h, 1, 5, L, 2.0, 0, 50.0, 0.0, 0.33, 0.25, warps, iters)
        f.copyImagesToDevice(pad_rows(I0, s), pad_rows(I1, s))
        f.solveOpticalFlow()
        u1, v1 = f.copyOpticalFlowToHost()
        assert_bitexact(u, u1, f"pair {i} u", region=(h, w))
        assert_bitexact(v, v1, f"pair {i} v", region=(h, w))


def test_batch_rejects_unsupported(rf):
    with pytest.raises(rf.RfError):
        rf.ReconFlowBatch([(64, 48)], 2, method=17)
    with pytest.raises(rf.RfError):
        rf.ReconFlowBatch([(64, 48), (8, 4)], 4, method=14)  # 8x4 cannot make 4 levels


def test_tile_shapes_do_not_change_results(rf):
    """rf_batch_set_tiles changes how pixels map to blocks, never a value;
    bad shapes are rejected; the autotuner leaves a valid choice."""
    from reconflow_gb300 import autotune
    from reconflow_gb300._native import RfError

    L = 3
    data = _inputs()
    kw = dict(lambda_=50.0, lambdaf=0.1, lambdams=100.0, alphaTv=1 / 0.33, alphaProj=60.0,
              tau=0.25, nWarpIters=2, nSolverIters=4, fix_quirks=1)
    b = rf.ReconFlowBatch([(w, h) for w, h, *_ in data], L, method=14, **kw)
    for i, (w, h, I0, I1, K, R, t) in enumerate(data):
        s = b.strides[i]
        b.setCameraMatrices(i, K, K)
        b.copyImagesToDevice(i, pad_rows(I0, s), pad_rows(I1, s))
    Rs, ts = [d[5] for d in data], [d[6] for d in data]
    b.solveR(Rs, ts)
    ref = [b.copyOpticalFlowToHost(i) + b.copy3dToHost(i) for i in range(len(data))]
    for tw, th in (([64, 16, 128], [4, 16, 2]), ([16, 32, 32], [8, 2, 4]), ([128, 64, 16], [2, 2, 2])):
        b.setTiles(tw, th)
        b.solveR(Rs, ts)
        for i in range(len(data)):
            got = b.copyOpticalFlowToHost(i) + b.copy3dToHost(i)
            for a, r, nm in zip(got, ref[i], "uvXYZ"):
                assert_bitexact(a, r, f"pair {i} {nm} tiles {tw}x{th}")
    for bad in (([0, 32, 32], [8, 8, 8]), ([32, 32, 33], [8, 8, 1]), ([64, 32, 32], [8, 8, 8])):
        with pytest.raises(RfError):
            b.setTiles(*bad)
    table = autotune.autotune(b, Rs, ts, iters=2)
    assert len(table) == L and all(tuple(e["tile"]) in autotune.CANDIDATES for e in table)
    tw, th = autotune.tiles_for(b, table)
    assert [tuple(x) for x in zip(tw, th)] == [tuple(e["tile"]) for e in table]
    b.close()


def test_bulk_transfers_match_per_pair_calls(rf):
    """rf_batch_upload_all / rf_batch_download_all move the same bytes as the
    per-pair calls (one pitch for every pair)."""
    import ctypes

    from reconflow_gb300 import _native

    lib = _native.load()
    sizes = [(64, 48), (50, 40), (64, 30)]
    pitch = 64
    kw = dict(lambda_=50.0, lambdaf=0.1, lambdams=100.0, alphaTv=1 / 0.33, alphaProj=60.0,
              tau=0.25, nWarpIters=1, nSolverIters=3, fix_quirks=1)
    b = rf.ReconFlowBatch(sizes, 2, method=14, **kw)
    imgs = []
    for i, (w, h) in enumerate(sizes):
        rng = np.random.default_rng(50 + i)
        I0, I1 = textured_pair(rng, h, w)
        imgs.append((pad_rows(I0, pitch), pad_rows(I1, pitch)))
        b.setCameraMatrices(i, _K(w, h), _K(w, h))
    b.uploadAll([a.ctypes.data for a, _ in imgs], [c.ctypes.data for _, c in imgs], pitch)
    R_, t_ = zip(*[_pose(i) for i in range(len(sizes))])
    b.solveR(list(R_), list(t_))
    outs = [[np.full((h, pitch), 7.0, np.float32) for _ in range(6)] for (w, h) in sizes]
    cols = [[outs[i][k].ctypes.data for i in range(len(sizes))] for k in range(6)]
    b.downloadAll(pitch, u=cols[0], v=cols[1], inv_depth=cols[2], X=cols[3], Y=cols[4],
                  Z=cols[5])
    for i, (w, h) in enumerate(sizes):
        u, v = b.copyOpticalFlowToHost(i)
        X, Y, Z = b.copy3dToHost(i)
        inv = b.copyInverseDepthToHost(i)
        for got, want, nm in zip(outs[i], (u, v, inv, X, Y, Z), ("u", "v", "inv", "X", "Y", "Z")):
            assert_bitexact(got[:, :w], want[:, :w], f"pair {i} {nm}")
    # a pair uploaded one at a time gives the same solve
    b2 = rf.ReconFlowBatch(sizes, 2, method=14, **kw)
    for i, (w, h) in enumerate(sizes):
        b2.setCameraMatrices(i, _K(w, h), _K(w, h))
        s = b2.strides[i]
        b2.copyImagesToDevice(i, imgs[i][0][:, :s] if s <= pitch else pad_rows(imgs[i][0], s),
                              imgs[i][1][:, :s] if s <= pitch else pad_rows(imgs[i][1], s))
    b2.solveR(list(R_), list(t_))
    for i, (w, h) in enumerate(sizes):
        assert_bitexact(b2.copyOpticalFlowToHost(i)[0][:, :w], outs[i][0][:, :w], f"pair {i}")
    b.close()
    b2.close()


def test_pipelined_transfers_match_blocking_calls(rf):
    """rf_batch_stage_upload / take_upload / stage_download / wait_download
    in a serving loop (next frames up and last results down while a solve
    runs, pinned host memory) give every step the bytes of a blocking
    upload_all + solve + download_all of the same frames."""
    import ctypes

    from reconflow_gb300 import _native

    lib = _native.load()
    sizes = [(64, 48), (50, 40), (64, 30)]
    pitch = 64
    kw = dict(lambda_=50.0, lambdaf=0.1, lambdams=100.0, alphaTv=1 / 0.33, alphaProj=60.0,
              tau=0.25, nWarpIters=1, nSolverIters=3, fix_quirks=1)
    R_, t_ = zip(*[_pose(i) for i in range(len(sizes))])
    held = []

    def pinned(h):
        p = ctypes.c_void_p()
        _native.check(lib.rf_host_alloc(h * pitch * 4, ctypes.byref(p)))
        held.append(p)
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_float)),
                                     shape=(h, pitch))

    frames = []  # two frame sets, [set][pair] = (I0, I1) in pinned memory
    for s in range(2):
        fs = []
        for i, (w, h) in enumerate(sizes):
            I0, I1 = textured_pair(np.random.default_rng(70 + 10 * s + i), h, w)
            a, c = pinned(h), pinned(h)
            a[:] = pad_rows(I0, pitch)
            c[:] = pad_rows(I1, pitch)
            fs.append((a, c))
        frames.append(fs)
    try:
        want = []
        ref = rf.ReconFlowBatch(sizes, 2, method=14, **kw)
        for i, (w, h) in enumerate(sizes):
            ref.setCameraMatrices(i, _K(w, h), _K(w, h))
        for fs in frames:
            ref.uploadAll([a.ctypes.data for a, _ in fs], [c.ctypes.data for _, c in fs], pitch)
            ref.solveR(list(R_), list(t_))
            outs = [[np.full((h, pitch), 7.0, np.float32) for _ in range(6)] for (w, h) in sizes]
            cols = [[outs[i][k].ctypes.data for i in range(len(sizes))] for k in range(6)]
            ref.downloadAll(pitch, u=cols[0], v=cols[1], inv_depth=cols[2], X=cols[3],
                            Y=cols[4], Z=cols[5])
            want.append(outs)
        ref.close()

        b = rf.ReconFlowBatch(sizes, 2, method=14, **kw)
        for i, (w, h) in enumerate(sizes):
            b.setCameraMatrices(i, _K(w, h), _K(w, h))
        with pytest.raises(Exception):
            b.takeUpload()  # nothing staged
        order = [0, 1, 0, 1]
        got = []
        b.stageUpload([a.ctypes.data for a, _ in frames[0]], [c.ctypes.data for _, c in frames[0]],
                      pitch)
        with pytest.raises(Exception):
            b.stageUpload([a.ctypes.data for a, _ in frames[0]],
                          [c.ctypes.data for _, c in frames[0]], pitch)  # staged twice
        for k, s in enumerate(order):
            b.takeUpload()
            if k + 1 < len(order):
                fs = frames[order[k + 1]]
                b.stageUpload([a.ctypes.data for a, _ in fs], [c.ctypes.data for _, c in fs], pitch)
            b.solveR(list(R_), list(t_))
            outs = [[pinned(h) for _ in range(6)] for (w, h) in sizes]
            for o in outs:
                for x in o:
                    x[:] = 7.0
            cols = [[outs[i][q].ctypes.data for i in range(len(sizes))] for q in range(6)]
            b.stageDownload(pitch, u=cols[0], v=cols[1], inv_depth=cols[2], X=cols[3], Y=cols[4],
                            Z=cols[5])
            got.append(outs)
        b.waitDownload()
        for k, s in enumerate(order):
            for i, (w, h) in enumerate(sizes):
                for q, nm in enumerate(("u", "v", "inv", "X", "Y", "Z")):
                    assert_bitexact(got[k][i][q][:, :w], want[s][i][q][:, :w],
                                    f"step {k} pair {i} {nm}")
        b.close()
    finally:
        for p in held:
            lib.rf_host_free(p)


def test_imported_results_replace_a_pair(rf):
    """rf_batch_import_results: a pair solved again by the single-pair solver
    (the learned path's fallback) and imported into the batch is what the
    batch downloads, bit for bit; the other pairs keep their own results."""
    ins = _inputs()[:2]
    kw = dict(method=14, lambda_=50.0, lambdaf=0.1, lambdams=100.0, alphaTv=1 / 0.33,
              alphaProj=60.0, tau=0.25, nWarpIters=1, nSolverIters=6, fix_quirks=1)
    b = rf.ReconFlowBatch([(w, h) for w, h, *_ in ins], 3, **kw)
    for i, (w, h, I0, I1, K, R, t) in enumerate(ins):
        b.setCameraMatrices(i, K, K)
        b.copyImagesToDevice(i, pad_rows(I0, b.strides[i]), pad_rows(I1, b.strides[i]))
    b.solveR([x[5] for x in ins], [x[6] for x in ins])
    keep = [b.copyOpticalFlowToHost(0)[0].copy()]
    # pair 1 solved alone with a longer schedule, then imported
    w, h, I0, I1, K, R, t = ins[1]
    f = rf.ReconFlow()
    f.initializeR(w, h, 1, 3, 2.0, 14, 50.0, 0.0, 0.1, 100.0, 1 / 0.33, 60.0, 0.5, 0.25, 2, 20,
                  cvType=5, fix_quirks=1)
    f.setCameraMatrices(K, K)
    f.copyImagesToDevice(pad_rows(I0, f.stride), pad_rows(I1, f.stride))
    f.solveR(R, t, 5.0)
    u1, v1 = f.copyOpticalFlowToHost()
    X1, Y1, Z1 = f.copy3dToHost()
    b.importResults(1, f.deviceResults(), f.stride)
    u, v = b.copyOpticalFlowToHost(1)
    X, Y, Z = b.copy3dToHost(1)
    for got, want, nm in ((u, u1, "u"), (v, v1, "v"), (X, X1, "X"), (Y, Y1, "Y"), (Z, Z1, "Z")):
        assert_bitexact(got[:, :w], want[:, :w], nm)
    assert_bitexact(b.copyOpticalFlowToHost(0)[0], keep[0], "pair 0 untouched")
    f.close()
    b.close()

"""CPU self-check of the network oracle: its analytic backward pass against
central finite differences of its forward pass (float64, BF16 rounding off);
and the committed checkpoint against the oracle's layer table."""
import numpy as np


def test_oracle_backward_matches_finite_differences():
    from oracle import cnn_oracle as CO

    CO.ROUND = False
    try:
        rng = np.random.default_rng(0)
        n = sum(co * 9 * ci + co for ci, co, _, _ in CO.LAYERS)
        params = rng.normal(0, 0.2, n)
        B, H, W = 1, 6, 5
        x = rng.normal(0, 1, (B, H, W, 16))
        t16 = rng.normal(0, 1, (B, 3, 3, 8))
        t8 = rng.normal(0, 1, (B, H, W, 8))
        m16 = np.ones((B, 3, 3))
        m8 = np.ones((B, H, W))
        # a smooth loss (L2) for finite differences: use pred - target as the
        # gradient by replacing L1 with a quadratic through the same code path
        g, loss, _ = CO.backward(params, x, t16, m16, t8, m8)

        def loss_of(p):
            return CO.backward(p, x, t16, m16, t8, m8)[1]

        eps = 1e-6
        idx = rng.choice(n, 40, replace=False)
        for i in idx:
            d = np.zeros(n)
            d[i] = eps
            num = (loss_of(params + d) - loss_of(params - d)) / (2 * eps)
            assert abs(num - g[i]) <= 1e-5 + 1e-3 * abs(num), (i, num, g[i])
    finally:
        CO.ROUND = True


def test_committed_checkpoint_matches_the_architecture(tmp_path):
    """The committed warm-start weights carry the checkpoint header (magic,
    version, parameter count, CRC32) and as many parameters as the layer
    table holds; a flipped byte or a wrong count is refused before any
    parameter reaches the network."""
    import os
    import shutil

    import pytest

    from oracle import cnn_oracle as CO
    from reconflow_gb300 import warmstart as WS
    from reconflow_gb300._native import RfError

    n = sum(co * 9 * ci + co for ci, co, _, _ in CO.LAYERS)
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "reconflow_gb300", "weights", "warmstart_f125.bin")

    class Net:  # the checkpoint reader needs only the count and a sink
        n_params = n
        got = None

        def set_params(self, p):
            self.got = p

    net = Net()
    WS.WarmStartNet.load(net, path)
    assert net.got is not None and net.got.size == n and np.all(np.isfinite(net.got))
    layers = CO.unpack(net.got.astype(np.float64))
    assert [W.shape for W, _ in layers] == [(co, 3, 3, ci) for ci, co, _, _ in CO.LAYERS]

    bad = tmp_path / "bad.bin"
    shutil.copy(path, bad)
    with open(bad, "r+b") as f:
        f.seek(1000)
        b = f.read(1)
        f.seek(1000)
        f.write(bytes([b[0] ^ 0x10]))
    net2 = Net()
    with pytest.raises(RfError):
        WS.WarmStartNet.load(net2, str(bad))
    assert net2.got is None
    net3 = Net()
    net3.n_params = n - 8
    with pytest.raises(RfError):
        WS.WarmStartNet.load(net3, path)

"""The numpy restatement of the network's backward pass against finite differences."""
import numpy as np

import gnn_reference as R


def _small_net(rng, fin=8, hid=6, layers=3):
    shapes = [(fin, hid)] + [(2 * hid, hid)] * layers + [(hid, 2)]
    ws = [rng.normal(size=s) * 0.5 for s in shapes]
    bs = [rng.normal(size=s[1]) * 0.1 for s in shapes]
    return ws, bs


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    n = 12
    ws, bs = _small_net(rng)
    x0 = rng.normal(size=(n, 8))
    nbr = rng.integers(-1, n, size=(n, 4))
    t = rng.normal(size=(n, 2))

    def loss(ws_, bs_):
        out, _ = R.forward(ws_, bs_, x0, nbr, round_bf16=False)
        return 0.5 * ((out - t) ** 2).sum()

    out, cache = R.forward(ws, bs, x0, nbr, round_bf16=False)
    grads = R.backward(cache, nbr, out - t)
    eps = 1e-6
    for li in range(len(ws)):
        for _ in range(4):
            i, j = rng.integers(ws[li].shape[0]), rng.integers(ws[li].shape[1])
            wp = [w.copy() for w in ws]
            wm = [w.copy() for w in ws]
            wp[li][i, j] += eps
            wm[li][i, j] -= eps
            fd = (loss(wp, bs) - loss(wm, bs)) / (2 * eps)
            assert abs(fd - grads[li][i, j]) <= 1e-6 * max(1.0, abs(fd))
        j = rng.integers(bs[li].shape[0])
        bp = [b.copy() for b in bs]
        bm = [b.copy() for b in bs]
        bp[li][j] += eps
        bm[li][j] -= eps
        fd = (loss(ws, bp) - loss(ws, bm)) / (2 * eps)
        assert abs(fd - grads[len(ws) + li][j]) <= 1e-6 * max(1.0, abs(fd))


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -9, 3.14159265, -2.5e-3])
    r = R.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0  # halfway and below: to even
    assert abs(r[3] - 3.140625) < 1e-12
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)

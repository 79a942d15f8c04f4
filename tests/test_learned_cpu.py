"""The numpy restatement of the network's backward pass against finite differences; the batched
feature builder against the per-sample one."""
import numpy as np
import torch

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


def test_batch_node_features_equal_per_sample(pkg):
    """The batched feature builder reproduces node_features column by column (values and
    neighbour ids shifted to each sample's first node)."""
    L = pkg.learned
    meshes = [pkg.meshes.star_shape(1, seed=3), pkg.meshes.icosphere(1), pkg.meshes.star_shape(2, seed=5)]
    gs = [L.edge_graph(torch.tensor(v, dtype=torch.float32), torch.tensor(f, dtype=torch.int32)) for v, f in meshes]
    nc = 2
    rng = np.random.default_rng(0)
    ks = [2.0, 3.5, 5.0]
    kh = rng.normal(size=(3, nc, 3))
    kh /= np.linalg.norm(kh, axis=2, keepdims=True)
    po = rng.normal(size=(3, nc, 3))
    nrows = max(g.n_edges for g in gs)
    B = torch.zeros(nrows, 3 * nc, dtype=torch.complex64)
    gen = torch.Generator().manual_seed(1)
    for i, g in enumerate(gs):
        B[:g.n_edges, i * nc:(i + 1) * nc] = torch.randn(g.n_edges, nc, dtype=torch.complex64, generator=gen)
    x0, nbr, flat = L.batch_node_features(L.batch_graph(gs), ks, kh, po, B, nc)
    off = 0
    for i, g in enumerate(gs):
        for r in range(nc):
            ref = L.node_features(g, ks[i], kh[i, r], po[i, r], B[:g.n_edges, i * nc + r])
            assert torch.allclose(ref.float(), x0[off:off + g.n_edges].float(), atol=1e-2, rtol=1e-2)
            nb = nbr[off:off + g.n_edges].long()
            assert torch.equal(torch.where(nb >= 0, nb - off, nb).int(), g.nbr)
            assert torch.equal(B.reshape(-1)[flat[off:off + g.n_edges]], B[:g.n_edges, i * nc + r])
            off += g.n_edges
    assert off == x0.shape[0]

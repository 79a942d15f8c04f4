"""The network's GPU kernels (forward, backward, Adam) against the numpy restatement, and a
training run that learns."""
import numpy as np
import pytest
import torch

import gnn_reference as R

pytestmark = pytest.mark.gpu


def _graph(pkg, cuda):
    v, f = pkg.meshes.star_shape(2, seed=7)
    return pkg.learned.edge_graph(torch.tensor(v, dtype=torch.float32, device=cuda),
                                  torch.tensor(f, dtype=torch.int32, device=cuda))


def test_edge_graph(pkg, cuda):
    g = _graph(pkg, cuda)
    nbr = g.nbr.cpu().numpy()
    assert nbr.shape == (g.n_edges, 4) and np.all(nbr >= 0)  # closed mesh: two triangles per edge
    assert np.all(nbr != np.arange(g.n_edges)[:, None])
    # symmetric: j is a neighbour of i iff i is a neighbour of j
    pairs = {(i, j) for i in range(g.n_edges) for j in nbr[i]}
    assert all((j, i) in pairs for i, j in pairs)


def test_forward_backward_match_reference(pkg, cuda):
    L = pkg.learned
    g = _graph(pkg, cuda)
    net = L.EdgeGNN(cuda, seed=1)
    rng = np.random.default_rng(0)
    # non-trivial biases so every path of the backward pass is exercised
    for b in net.b:
        b.copy_(torch.tensor(rng.normal(size=b.shape) * 0.05, dtype=torch.float32))
    b_e = torch.complex(torch.randn(g.n_edges), torch.randn(g.n_edges)).to(cuda)
    x0 = L.node_features(g, 4.0, [0, 0, 1.0], [1.0, 0, 0], b_e)
    out, cache = net.forward(x0, g.nbr)
    t = torch.randn_like(out)
    dout = (out - t) * (2.0 / out.shape[0])
    grads = net.backward(cache, dout)
    ws = [w.double().cpu().numpy() for w in net.w]
    bs = [b.double().cpu().numpy() for b in net.b]
    x0n = x0.float().cpu().numpy().astype(np.float64)
    nbr = g.nbr.cpu().numpy()
    ref_out, rcache = R.forward(ws, bs, x0n, nbr)
    rel = lambda a, b: np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)  # noqa: E731
    assert rel(out.cpu().numpy(), ref_out) < 2e-2
    ref_grads = R.backward(rcache, nbr, dout.double().cpu().numpy())
    for i, (gg, rg) in enumerate(zip(grads, ref_grads)):
        assert rel(gg.double().cpu().numpy(), rg) < 5e-2, i


def test_adam_and_training_reduce_loss(pkg, cuda):
    L = pkg.learned
    g = _graph(pkg, cuda)
    items = []
    rng = np.random.default_rng(1)
    for s in range(16):
        b_e = torch.complex(torch.randn(g.n_edges), torch.randn(g.n_edges)).to(cuda)
        khat = rng.normal(size=3)
        khat /= np.linalg.norm(khat)
        x0 = L.node_features(g, 3.0, khat, np.cross(khat, [0.3, 0.4, 0.5]), b_e)
        # a local, learnable target: J = b smoothed over the neighbours
        nb = g.nbr.long()
        j = 0.5 * b_e + 0.125 * b_e[nb].sum(1)
        items.append((g, x0, j))
    samples = L.build_samples(items)
    net = L.EdgeGNN(cuda, seed=0)
    losses = L.train(net, samples, epochs=30, batch=4, lr=2e-3)
    assert losses[-1] < 0.5 * losses[0], losses

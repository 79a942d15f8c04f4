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


def test_subspace_guess_beats_scaled_prediction(pkg, cuda):
    """The least-squares guess over a mesh's prediction subspace has a residual no larger than
    the best multiple of the column's own prediction (which the subspace contains), and keeps
    rows beyond E_i at zero; the solver started from it converges and reports per-column
    Arnoldi steps."""
    L, M = pkg.learned, pkg.meshes
    meshes = [M.star_shape(2, seed=11), M.icosphere(1), M.star_shape(2, seed=12)]
    ks = [2.0, 3.0, 4.0]
    bt = pkg.batch.MeshBatch(meshes, ks, device=cuda, formulation="cfie_ref")
    nc = 4
    rng = np.random.default_rng(3)
    waves = []
    for i in range(bt.n_mesh):
        d = rng.normal(size=(nc, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        p = np.cross(d, rng.normal(size=(nc, 3)))
        waves.append(pkg.mesh_MOM_3d.plane_waves(ks[i], d, p))
    Z = bt.assemble()
    B = bt.excitation(torch.stack(waves).to(cuda))
    X, info = bt.solve(Z, B, restart=50, tol=1e-6, max_iters=500)
    # a noisy "prediction": the solution plus 30 % noise
    gen = torch.Generator(device="cpu").manual_seed(0)
    noise = torch.randn(X.shape, dtype=torch.complex128, generator=gen).to(cuda)
    for i in range(bt.n_mesh):
        noise[bt.n_edges[i]:, i * nc:(i + 1) * nc] = 0
    Pm = (X + 0.3 * noise * X.abs().mean()).to(torch.complex64)
    flat = torch.cat([torch.arange(bt.n_edges[i], device=cuda)[None, :].repeat(nc, 1).reshape(-1) * B.shape[1]
                      + torch.arange(i * nc, (i + 1) * nc, device=cuda).repeat_interleave(bt.n_edges[i])
                      for i in range(bt.n_mesh)])
    pred = Pm.reshape(-1)[flat]
    X0 = L.subspace_guess(bt, Z, B, pred, flat, nc)
    r_ls = torch.linalg.norm((bt.matvec(Z, X0.to(torch.complex64)) - B).to(torch.complex128), dim=0)
    zp = bt.matvec(Z, Pm).to(torch.complex128)
    alpha = (zp.conj() * B).sum(0) / (zp.abs() ** 2).sum(0)
    r_sc = torch.linalg.norm(zp * alpha - B, dim=0)
    assert torch.all(r_ls <= r_sc * (1 + 1e-3) + 1e-6), (r_ls, r_sc)
    for i in range(bt.n_mesh):
        assert torch.all(X0[bt.n_edges[i]:, i * nc:(i + 1) * nc] == 0)
    X1, info1 = bt.solve(Z, B, restart=50, tol=1e-6, max_iters=500, X0=X0)
    assert info1["converged"]
    cs = info1["column_iterations"].cpu()
    assert cs.shape[0] == B.shape[1] and int(cs.max()) <= info1["iterations"]
    assert float(cs.double().mean()) <= 1.02 * float(info["column_iterations"].double().mean())

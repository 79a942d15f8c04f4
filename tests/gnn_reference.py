"""Float64 numpy restatement of the edge-graph network (test infrastructure): forward and
backward with the same BF16 rounding of weights and activations as the GPU kernels, so the
kernels' outputs and gradients can be compared against it; the backward itself is checked
against finite differences on the CPU."""
import numpy as np


def bf16(x):
    """Round to bfloat16 (nearest even), returned as float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    u = (u + np.uint32(0x7FFF) + ((u >> np.uint32(16)) & np.uint32(1))) & np.uint32(0xFFFF0000)
    return u.view(np.float32).astype(np.float64)


def aggregate(h, nbr):
    out = np.zeros_like(h)
    deg = (nbr >= 0).sum(1)
    for j in range(nbr.shape[1]):
        q = nbr[:, j]
        ok = q >= 0
        out[ok] += h[q[ok]]
    out[deg > 0] /= deg[deg > 0, None]
    return np.concatenate([h, out], 1)


def aggregate_bwd(dcat, nbr):
    f = dcat.shape[1] // 2
    dh = dcat[:, :f].copy()
    deg = (nbr >= 0).sum(1)
    g = np.zeros_like(dh)
    g[deg > 0] = dcat[deg > 0, f:] / deg[deg > 0, None]
    for j in range(nbr.shape[1]):
        q = nbr[:, j]
        ok = q >= 0
        np.add.at(dh, q[ok], g[ok])
    return dh


def forward(ws, bs, x0, nbr, round_bf16=True):
    r = bf16 if round_bf16 else (lambda a: a)
    ws = [r(w) for w in ws]
    h = r(np.maximum(r(x0) @ ws[0] + bs[0], 0))
    hs, cats = [h], []
    for layer in range(1, len(ws) - 1):
        cat = r(aggregate(h, nbr))
        cats.append(cat)
        h = r(np.maximum(cat @ ws[layer] + bs[layer], 0))
        hs.append(h)
    out = h @ ws[-1] + bs[-1]
    return out, (r(x0), ws, hs, cats)


def backward(cache, nbr, dout):
    x0, ws, hs, cats = cache
    gw = [None] * len(ws)
    gb = [None] * len(ws)
    gw[-1] = hs[-1].T @ dout
    gb[-1] = dout.sum(0)
    dh = dout @ ws[-1].T
    for layer in range(len(ws) - 2, 0, -1):
        dz = dh * (hs[layer] > 0)
        gw[layer] = cats[layer - 1].T @ dz
        gb[layer] = dz.sum(0)
        dh = aggregate_bwd(dz @ ws[layer].T, nbr)
    dz = dh * (hs[0] > 0)
    gw[0] = x0.T @ dz
    gb[0] = dz.sum(0)
    return gw + gb

"""CPU checks of the symmetric-rule EFIE path's mathematics (oracle side).

* The closed-form potential integrals (Wilton et al. 1984) against brute-force quadrature.
* The oracle's 7-point-rule EFIE with singularity extraction against the Mie series for
  the PEC sphere (tests/mie.py): the surface current converges at first order.
"""
import numpy as np
import pytest
import torch

import mie
from conftest import rel_err


def _brute_potential(x, P, n=300):
    """int_T 1/R and int_T (y - x)/R by splitting T at the projection of x (no Duffy)."""
    g, w = np.polynomial.legendre.leggauss(n)
    g, w = (g + 1) / 2, w / 2
    U, V = np.meshgrid(g, g, indexing="ij")
    W = np.outer(w, w)
    r1, r2 = U, U * V
    nrm = np.cross(P[1] - P[0], P[2] - P[1])
    nrm /= np.linalg.norm(nrm)
    rho = x - np.dot(x - P[0], nrm) * nrm
    i1, iv = 0.0, np.zeros(3)
    for i in range(3):
        a, b = P[i], P[(i + 1) % 3]
        As = 0.5 * np.dot(np.cross(a - rho, b - rho), nrm)
        y = (1 - r1)[..., None] * rho + (r1 - r2)[..., None] * a + r2[..., None] * b
        R = np.linalg.norm(y - x, axis=-1)
        wt = W * U * 2 * As
        i1 += np.sum(wt / R)
        iv += np.sum((wt / R)[..., None] * (y - x), axis=(0, 1))
    return i1, iv


def test_potential_integrals_closed_form(oracle):
    P = np.array([[0.0, 0, 0], [1, 0.1, 0], [0.3, 0.9, 0.05]])
    n = np.cross(P[1] - P[0], P[2] - P[1])
    n /= np.linalg.norm(n)
    pts = [P.mean(0), P.mean(0) + 0.3 * n, np.array([2.0, 1.5, 0.4]), 0.2 * P[0] + 0.5 * P[1] + 0.3 * P[2],
           0.6 * P[0] + 0.2 * P[1] + 0.2 * P[2] - 0.05 * n, P[0] + 0.5 * (P[1] - P[0]) + 0.2 * n,
           P[1] + 0.3 * (P[1] - P[2]) + 0.01 * n]
    for x in pts:
        a1, av = oracle.potential_integrals(x, P)
        b1, bv = _brute_potential(x, P)
        assert abs(a1 - b1) / abs(b1) < 1e-12
        assert np.linalg.norm(av - bv) / np.linalg.norm(bv) < 1e-11


def test_mie_series_self_consistent():
    for k in (0.5, 2.0, 10.0):
        pw, tang = mie.self_check(k=k)
        assert pw < 1e-9 and tang < 1e-12


def _face_centroid_current(v, f, fei, I):
    P = v[f]
    c = P.mean(1)
    A = 0.5 * np.linalg.norm(np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 1]), axis=1)
    J = np.zeros((f.shape[0], 3), complex)
    for e in range(3):
        i1, i2 = f[:, (e + 1) % 3], f[:, (e + 2) % 3]
        l = np.linalg.norm(P[:, (e + 2) % 3] - P[:, (e + 1) % 3], axis=1)
        s = np.where(i1 < i2, 1.0, -1.0) * l / (2 * A)
        J += (s * I[fei.reshape(-1, 3)[:, e]])[:, None] * (c - P[:, e])
    return c, J


def test_symmetric_efie_converges_to_mie(pkg, oracle):
    errs = []
    k = 2.0
    for level in (1, 2, 3):
        v, f = pkg.meshes.icosphere(level)
        edges, fei, _ = pkg.utils.get_edge_unique(torch.tensor(v), torch.tensor(f))
        fei = fei.numpy()
        ne = edges.shape[0]
        Z = oracle.mom_sym_zmat(v, f, fei, ne, k)
        b = oracle.mom_sym_rhs(v, f, fei, ne, np.array([[0, 0, k, 1, 0, 0, 0, 1, 0]], float))[:, 0]
        c, J = _face_centroid_current(v, f, fei, np.linalg.solve(Z, b))
        errs.append(rel_err(J, mie.surface_current(c, k, 1.0)))
    assert errs[2] < 0.05
    assert errs[1] < 0.6 * errs[0] and errs[2] < 0.6 * errs[1]

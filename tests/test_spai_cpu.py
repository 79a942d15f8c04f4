"""CPU checks of the preconditioner's numpy restatement (spai_reference.py) on the oracle's
7-point EFIE matrix: the patterns are symmetric and nested, and M improves the spectrum."""
import numpy as np

import spai_reference as SR


def _efie_l1(pkg, oracle, k=2.0):
    import torch

    v, f = pkg.meshes.icosphere(1)
    vt, ft = torch.tensor(v, dtype=torch.float32), torch.tensor(f)
    edges, fei, _ = pkg.utils.get_edge_unique(vt, ft)
    ne = edges.shape[0]
    fei = fei.numpy().reshape(-1)
    Z = oracle.mom_sym_zmat(vt.double().numpy(), f, fei, ne, k)
    return f, fei, ne, Z


def test_patterns_are_symmetric_and_nested(pkg, oracle):
    f, fei, ne, _ = _efie_l1(pkg, oracle)
    pats = SR.patterns(f, fei, ne)
    for j, (J, I) in enumerate(pats):
        assert j in J and set(J) <= set(I)
        assert J.size <= 48 and I.size <= 128
        for i in J:
            assert j in pats[int(i)][0]


def test_restated_preconditioner_improves_conditioning(pkg, oracle):
    f, fei, ne, Z = _efie_l1(pkg, oracle)
    M = SR.dense_m(SR.spai_columns(Z, SR.patterns(f, fei, ne)), ne)
    s0 = np.linalg.svd(Z, compute_uv=False)
    s1 = np.linalg.svd(Z @ M, compute_uv=False)
    assert s1[0] / s1[-1] < 0.5 * s0[0] / s0[-1]
    # each column's fit beats m = 0 (residual 1)
    R = Z @ M - np.eye(ne)
    assert (np.linalg.norm(R, axis=0) < 1.0).all()

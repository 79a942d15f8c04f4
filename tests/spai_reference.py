"""numpy restatement of the near-field sparse approximate inverse (csrc/spai.cu), the
checker of its GPU tests.  Column j of M minimises ||Z[I_j, J_j] m - e_j|| (least squares
in complex128) with J_j the edges of the faces that share a vertex with a face of edge j,
and I_j the edges of the faces that share a vertex with a face of J_j.  Meshes here stay
below the kernel's caps (48 columns, 128 rows), so no pattern is cut."""
import numpy as np


def vertex_neighbour_faces(faces):
    """N(f): sorted faces sharing at least one vertex with f (f included)."""
    vf = {}
    for f, tri in enumerate(faces):
        for v in tri:
            vf.setdefault(int(v), set()).add(f)
    return [sorted(set().union(*(vf[int(v)] for v in tri))) for tri in faces]


def patterns(faces, fei, n_edges):
    fe = np.asarray(fei).reshape(-1, 3)
    nbr = vertex_neighbour_faces(np.asarray(faces))
    ef = [[] for _ in range(n_edges)]
    for f in range(fe.shape[0]):
        for e in fe[f]:
            ef[int(e)].append(f)
    out = []
    for j in range(n_edges):
        s1 = sorted(set().union(*(nbr[f] for f in ef[j])))
        J = np.unique(fe[s1].reshape(-1))
        s2 = sorted(set().union(*(nbr[g] for g in s1)))
        I = np.unique(fe[s2].reshape(-1))
        out.append((J, I))
    return out


def spai_columns(Z, pats):
    """{j: (J_j, m_j)} with m_j the complex128 least-squares solution."""
    cols = {}
    for j, (J, I) in enumerate(pats):
        A = Z[np.ix_(I, J)].astype(np.complex128)
        e = (I == j).astype(np.complex128)
        cols[j] = (J, np.linalg.lstsq(A, e, rcond=None)[0])
    return cols


def dense_m(cols, n):
    M = np.zeros((n, n), np.complex128)
    for j, (J, m) in cols.items():
        M[J, j] = m
    return M

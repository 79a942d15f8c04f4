"""Batched meshes: one launch assembles / excites every mesh; lockstep GMRES on the block-
diagonal system (with and without the captured CUDA graph) against per-mesh results."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _bipyramid():
    """Pentagonal bipyramid: 7 vertices, 10 faces, 15 edges (an odd edge count, so its Z
    block has padded rows)."""
    a = 2 * np.pi * np.arange(5) / 5
    v = np.concatenate([np.stack([np.cos(a), np.sin(a), np.zeros(5)], 1), [[0, 0, 1.2], [0, 0, -1.2]]])
    f = [[k, (k + 1) % 5, 5] for k in range(5)] + [[(k + 1) % 5, k, 6] for k in range(5)]
    return v.astype(np.float32), np.asarray(f, np.int32)


def _batch(pkg, cuda):
    M = pkg.meshes
    meshes = [M.icosphere(1, 1.0), _bipyramid(), M.ellipsoid(2), M.star_shape(2, seed=3)]
    ks = [1.5, 2.0, 2.5, 3.0]
    return pkg.batch.MeshBatch(meshes, ks, device=cuda), meshes, ks


def _waves(pkg, n_mesh, nc, ks, cuda, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_mesh):
        d = rng.normal(size=(nc, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        p = np.cross(d, rng.normal(size=(nc, 3)))
        p /= np.linalg.norm(p, axis=1, keepdims=True)
        out.append(pkg.mesh_MOM_3d.plane_waves(ks[i], d, p))
    return torch.stack(out).to(cuda)


def _per_mesh(pkg, cuda, v, f, k, waves):
    MM = pkg.mesh_MOM_3d
    vt = torch.tensor(np.asarray(v), dtype=torch.float32, device=cuda)
    ft = torch.tensor(np.asarray(f), dtype=torch.int32, device=cuda)
    edges, fei, _ = pkg.utils.get_edge_unique(vt, ft)
    Z = MM.assemble_Z_rwg_sym(vt, ft, fei, edges.shape[0], k)
    B = MM.assemble_rhs_rwg_sym(vt, ft, fei, edges.shape[0], waves)
    return Z, B


def test_batched_assembly_and_excitation_match_per_mesh(pkg, cuda):
    bt, meshes, ks = _batch(pkg, cuda)
    waves = _waves(pkg, bt.n_mesh, 4, ks, cuda)
    Z = bt.assemble()
    B = bt.excitation(waves)
    for i, (v, f) in enumerate(meshes):
        Zi, Bi = _per_mesh(pkg, cuda, v, f, ks[i], waves[i])
        zb = bt.z_block(Z, i)
        assert (torch.linalg.norm(zb - Zi) / torch.linalg.norm(Zi)).item() < 1e-6
        for r in range(4):
            bc = bt.column(B, i, r)
            assert (torch.linalg.norm(bc - Bi[:, r]) / torch.linalg.norm(Bi[:, r])).item() < 1e-6
        assert torch.all(B[bt.n_edges[i]:, 4 * i:4 * i + 4] == 0)


@pytest.mark.parametrize("nc", [1, 4])
@pytest.mark.parametrize("rows", [1, 2, 4, 8, 32])
def test_blockdiag_matvec(pkg, cuda, nc, rows):
    bt, meshes, ks = _batch(pkg, cuda)
    bt.excitation(_waves(pkg, bt.n_mesh, nc, ks, cuda))
    Z = bt.assemble()
    g = torch.Generator(device="cpu").manual_seed(rows * 10 + nc)
    X = torch.randn(bt.n_rows, bt.n_mesh * nc, dtype=torch.complex64, generator=g).to(cuda)
    for i in range(bt.n_mesh):
        X[bt.n_edges[i]:, i * nc:(i + 1) * nc] = 0
    Y = bt.matvec(Z, X, rows)
    for i in range(bt.n_mesh):
        e = bt.n_edges[i]
        ref = bt.z_block(Z, i).to(torch.complex128) @ X[:e, i * nc:(i + 1) * nc].to(torch.complex128)
        got = Y[:e, i * nc:(i + 1) * nc].to(torch.complex128)
        assert (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item() < 1e-5
        assert torch.all(Y[e:, i * nc:(i + 1) * nc] == 0)


@pytest.mark.parametrize("use_graph,rows", [(False, None), (True, None), (True, 32)])
def test_batched_solve_matches_dense(pkg, cuda, use_graph, rows):
    bt, meshes, ks = _batch(pkg, cuda)
    waves = _waves(pkg, bt.n_mesh, 4, ks, cuda, seed=1)
    Z = bt.assemble()
    B = bt.excitation(waves)
    if rows is None:
        bt.autotune(Z)
    else:
        bt.rows_per_warp = rows
    X, info = bt.solve(Z, B, restart=50, tol=1e-6, max_iters=3000, use_graph=use_graph)
    assert info["converged"], info
    for i in range(bt.n_mesh):
        Zi = bt.z_block(Z, i).to(torch.complex128)
        e = bt.n_edges[i]
        ref = torch.linalg.solve(Zi, B[:e, 4 * i:4 * i + 4].to(torch.complex128))
        got = X[:e, 4 * i:4 * i + 4]
        err = (torch.linalg.norm(got - ref, dim=0) / torch.linalg.norm(ref, dim=0)).max().item()
        assert err < 1e-3, (i, err)
        assert torch.all(X[e:, 4 * i:4 * i + 4] == 0)


def test_batched_reference_cfie_matches_per_mesh_and_solves(pkg, cuda):
    M = pkg.meshes
    meshes = [M.icosphere(1, 1.0), M.star_shape(2, seed=5), M.ellipsoid(1)]
    ks = [2.0, 4.0, 3.0]
    bt = pkg.batch.MeshBatch(meshes, ks, device=cuda, formulation="cfie_ref")
    waves = _waves(pkg, bt.n_mesh, 4, ks, cuda, seed=2)
    Z = bt.assemble()
    B = bt.excitation(waves)
    MM, U = pkg.mesh_MOM_3d, pkg.utils
    px, wx = U.get_gaussion_integration_points_and_weights(4, device=cuda)
    py, wy = U.get_gaussion_integration_points_and_weights(3, device=cuda)
    for i, (v, f) in enumerate(meshes):
        vt = torch.tensor(np.asarray(v), dtype=torch.float32, device=cuda)
        ft = torch.tensor(np.asarray(f), dtype=torch.int32, device=cuda)
        edges, fei, _ = U.get_edge_unique(vt, ft)
        a, n = U.compute_face_areas(vt, ft).contiguous(), U.compute_face_normals(vt, ft).contiguous()
        Zi = MM.assemble_Z_rwg(vt, ft, a, n, fei, edges.shape[0], px, wx, py, wy, ks[i])
        Bi = MM.assemble_rhs_rwg(vt, ft, a, n, fei, edges.shape[0], px, wx, waves[i])
        assert (torch.linalg.norm(bt.z_block(Z, i) - Zi) / torch.linalg.norm(Zi)).item() < 1e-6
        got = B[: bt.n_edges[i], 4 * i:4 * i + 4]
        assert (torch.linalg.norm(got - Bi) / torch.linalg.norm(Bi)).item() < 1e-6
    bt.autotune(Z)
    X, info = bt.solve(Z, B, restart=50, tol=1e-6, max_iters=500, use_graph=True)
    assert info["converged"] and info["iterations"] <= 200
    for i in range(bt.n_mesh):
        e = bt.n_edges[i]
        ref = torch.linalg.solve(bt.z_block(Z, i).to(torch.complex128), B[:e, 4 * i:4 * i + 4].to(torch.complex128))
        err = (torch.linalg.norm(X[:e, 4 * i:4 * i + 4] - ref, dim=0) / torch.linalg.norm(ref, dim=0)).max().item()
        assert err < 1e-4, (i, err)


def test_batch_spai_equals_per_mesh_spai(pkg, cuda):
    """The near-field preconditioner built over the whole batch (one launch, flat Z with even
    row pitches, global near-pair list) equals the one built for each mesh alone."""
    bt, meshes, ks = _batch(pkg, cuda)
    bt.excitation(_waves(pkg, bt.n_mesh, 4, ks, cuda))
    Z = bt.assemble()
    P = bt.spai(Z)
    assert P.status == 0
    MM = pkg.mesh_MOM_3d
    for i, (v, f) in enumerate(meshes):
        vt = torch.tensor(np.asarray(v), dtype=torch.float32, device=cuda)
        ft = torch.tensor(np.asarray(f), dtype=torch.int32, device=cuda)
        edges, fei, _ = pkg.utils.get_edge_unique(vt, ft)
        e = edges.shape[0]
        Pi = MM.spai_preconditioner(bt.z_block(Z, i).contiguous(), vt, ft, fei, e)
        o = int(bt.edge_offsets[i])
        assert torch.equal(P.cols[o:o + e], Pi.cols)
        assert torch.equal(P.vals[o:o + e], Pi.vals)


@pytest.mark.parametrize("use_graph", [False, True])
def test_batched_preconditioned_solve_matches_dense(pkg, cuda, use_graph):
    bt, meshes, ks = _batch(pkg, cuda)
    waves = _waves(pkg, bt.n_mesh, 4, ks, cuda, seed=1)
    Z = bt.assemble()
    B = bt.excitation(waves)
    bt.autotune(Z)
    P = bt.spai(Z)
    # tol 1e-9: reachable only because each cycle of the preconditioned path starts from a
    # compensated (FP64-class) residual; the plain lockstep path's FP32 residual stops ~1e-6
    X, info = bt.solve(Z, B, restart=50, tol=1e-9, max_iters=3000, use_graph=use_graph, M=P)
    X0, info0 = bt.solve(Z, B, restart=50, tol=1e-6, max_iters=3000, use_graph=use_graph)
    assert info["converged"], info
    assert info["iterations"] < 2 * info0["iterations"]
    steps = info["column_iterations"].cpu().numpy()
    assert steps.max() <= info["iterations"]
    for i in range(bt.n_mesh):
        Zi = bt.z_block(Z, i).to(torch.complex128)
        e = bt.n_edges[i]
        ref = torch.linalg.solve(Zi, B[:e, 4 * i:4 * i + 4].to(torch.complex128))
        got = X[:e, 4 * i:4 * i + 4]
        err = (torch.linalg.norm(got - ref, dim=0) / torch.linalg.norm(ref, dim=0)).max().item()
        assert err < 1e-6, (i, err)
        assert torch.all(X[e:, 4 * i:4 * i + 4] == 0)


def test_batched_rows_assembly_every_tile_and_schedule(pkg, cuda):
    """The rows layout (8 / 16 / 32 test faces per block, meshes in packing order or largest
    first) assembles the same matrices as the one-pair-per-thread kernel; the autotuner picks
    one of them."""
    bt, meshes, ks = _batch(pkg, cuda)
    bt.excitation(_waves(pkg, bt.n_mesh, 4, ks, cuda))
    ref = bt.assemble()
    for cfg in [(r, o) for r in (8, 16, 32) for o in ("packed", "largest")]:
        bt.asm_config = cfg
        Z = bt.assemble()
        for i in range(bt.n_mesh):
            zi, zr = bt.z_block(Z, i), bt.z_block(ref, i)
            assert (torch.linalg.norm(zi - zr) / torch.linalg.norm(zr)).item() < 1e-6, (cfg, i)
    best = bt.autotune_assembly()
    assert best in [("pair", None)] + [(r, o) for r in (8, 16, 32) for o in ("packed", "largest")]
    Z = bt.assemble()
    assert (torch.linalg.norm(Z - ref) / torch.linalg.norm(ref)).item() < 1e-6


def test_batched_cfie_persistent_assembly_equals_grid(pkg, cuda):
    """The reference-rule batch assembled by the resident grid that takes its tiles from a
    work counter equals the one-block-per-tile launch (the same entries, summed by the same
    atomics: equal to 1e-6), on every mesh; the autotuner picks one of the two."""
    M = pkg.meshes
    meshes = [M.icosphere(1, 1.0), _bipyramid(), M.ellipsoid(2), M.star_shape(2, seed=3)]
    ks = [1.5, 2.0, 2.5, 3.0]
    bt = pkg.batch.MeshBatch(meshes, ks, device=cuda, formulation="cfie_ref")
    bt.excitation(_waves(pkg, bt.n_mesh, 4, ks, cuda))
    bt.asm_config = ("grid", None)
    ref = bt.assemble()
    bt.asm_config = ("persistent", None)
    for _ in range(2):  # the counter starts from zero on every call
        Z = bt.assemble()
        for i in range(bt.n_mesh):
            zi, zr = bt.z_block(Z, i), bt.z_block(ref, i)
            assert (torch.linalg.norm(zi - zr) / torch.linalg.norm(zr)).item() < 1e-6, i
    best = bt.autotune_assembly()
    assert best in [("grid", None), ("persistent", None)] and set(bt.asm_times) == {("grid", None),
                                                                                    ("persistent", None)}


def _dense_refs(bt, Z, B, nc=4):
    refs = []
    for i in range(bt.n_mesh):
        e = bt.n_edges[i]
        refs.append(torch.linalg.solve(bt.z_block(Z, i).to(torch.complex128), B[:e, nc * i:nc * (i + 1)].to(
            torch.complex128)))
    return refs


@pytest.mark.parametrize("k,precond,use_graph", [(8, False, False), (16, True, True), (4, True, False)])
def test_augmented_solve_matches_dense(pkg, cuda, k, precond, use_graph):
    """Lockstep GMRES with a random K-vector deflation subspace per mesh (with and without the
    near-field preconditioner, graph-captured or not) converges to the dense solution; the
    reported residual is the true one.  The preconditioned path starts its cycles from a
    compensated residual and reaches 1e-9; the plain lockstep path's FP32 cycle-start residual
    stalls near 1e-7, so it is asked for 1e-6."""
    bt, meshes, ks = _batch(pkg, cuda)
    waves = _waves(pkg, bt.n_mesh, 4, ks, cuda, seed=1)
    Z = bt.assemble()
    B = bt.excitation(waves)
    g = torch.Generator(device="cpu").manual_seed(3)
    U = torch.randn(bt.n_rows, bt.n_mesh, k, dtype=torch.complex64, generator=g).to(cuda)
    aug = bt.augmentation(Z, U)
    P = bt.spai(Z) if precond else None
    tol, err_max, res_max = (1e-9, 1e-5, 1e-8) if precond else (1e-6, 1e-3, 2e-6)
    X, info = bt.solve(Z, B, restart=30, tol=tol, max_iters=3000, use_graph=use_graph, M=P, aug=aug)
    assert info["converged"], info
    refs = _dense_refs(bt, Z, B)
    for i in range(bt.n_mesh):
        e = bt.n_edges[i]
        got = X[:e, 4 * i:4 * i + 4]
        err = (torch.linalg.norm(got - refs[i], dim=0) / torch.linalg.norm(refs[i], dim=0)).max().item()
        assert err < err_max, (i, err)
        assert torch.all(X[e:, 4 * i:4 * i + 4] == 0)
        r = B[:e, 4 * i:4 * i + 4].to(torch.complex128) - bt.z_block(Z, i).to(torch.complex128) @ got
        rel = (torch.linalg.norm(r, dim=0) / torch.linalg.norm(B[:e, 4 * i:4 * i + 4].to(torch.complex128),
                                                                 dim=0)).max().item()
        assert rel < res_max, (i, rel)


def test_augmented_subspace_holding_the_solutions_needs_no_arnoldi_step(pkg, cuda):
    """When each mesh's subspace holds its columns' solutions (real and imaginary parts of the
    four dense solutions: K = 8), the first cycle start already solves every column: no
    Arnoldi step is taken and the answer equals the dense one."""
    bt, meshes, ks = _batch(pkg, cuda)
    waves = _waves(pkg, bt.n_mesh, 4, ks, cuda, seed=4)
    Z = bt.assemble()
    B = bt.excitation(waves)
    refs = _dense_refs(bt, Z, B)
    U = torch.zeros(bt.n_rows, bt.n_mesh, 8, dtype=torch.complex64, device=cuda)
    for i in range(bt.n_mesh):
        e = bt.n_edges[i]
        U[:e, i, :4] = refs[i].real.to(torch.complex64)
        U[:e, i, 4:] = refs[i].imag.to(torch.complex64)
    X, info = bt.solve(Z, B, restart=20, tol=1e-5, max_iters=100, use_graph=False, aug=bt.augmentation(Z, U))
    assert info["converged"] and info["iterations"] == 0, info
    for i in range(bt.n_mesh):
        e = bt.n_edges[i]
        err = (torch.linalg.norm(X[:e, 4 * i:4 * i + 4] - refs[i], dim=0) / torch.linalg.norm(refs[i], dim=0))
        assert err.max().item() < 1e-5, (i, err)


def test_augmented_solve_rejects_bad_subspace(pkg, cuda):
    bt, meshes, ks = _batch(pkg, cuda)
    Z = bt.assemble()
    bt.excitation(_waves(pkg, bt.n_mesh, 4, ks, cuda))
    with pytest.raises(ValueError):
        bt.augmentation(Z, torch.zeros(bt.n_rows, bt.n_mesh, 5, dtype=torch.complex64, device=cuda))
    q, ut, k = bt.augmentation(Z, torch.ones(bt.n_rows, bt.n_mesh, 4, dtype=torch.complex64, device=cuda))
    B = bt.excitation(_waves(pkg, bt.n_mesh, 4, ks, cuda))
    with pytest.raises(ValueError):
        bt.solve(Z, B, aug=(q[:, :-1], ut[:, :-1], k))


@pytest.mark.parametrize("use_graph", [False, True])
def test_batched_solve_with_an_idle_mesh(pkg, cuda, use_graph):
    """A mesh whose right-hand sides are zero is inactive from the first cycle, so the
    Arnoldi products skip it throughout: its solution stays exactly zero and the other meshes
    still match the dense solve (with and without the preconditioner)."""
    bt, meshes, ks = _batch(pkg, cuda)
    waves = _waves(pkg, bt.n_mesh, 4, ks, cuda, seed=5)
    Z = bt.assemble()
    B = bt.excitation(waves)
    B[:, 4:8] = 0  # mesh 1
    refs = _dense_refs(bt, Z, B)
    for P in (None, bt.spai(Z)):
        X, info = bt.solve(Z, B, restart=40, tol=1e-6 if P is None else 1e-9, max_iters=3000,
                           use_graph=use_graph, M=P)
        assert info["converged"], info
        assert torch.all(X[:, 4:8] == 0)
        assert int(info["column_iterations"][4:8].max()) == 0
        for i in (0, 2, 3):
            e = bt.n_edges[i]
            got = X[:e, 4 * i:4 * i + 4]
            err = (torch.linalg.norm(got - refs[i], dim=0) / torch.linalg.norm(refs[i], dim=0)).max().item()
            assert err < (1e-3 if P is None else 1e-6), (i, err)

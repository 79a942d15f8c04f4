"""GPU symmetric-rule Laplace operators, the hypersingular operator and the Neumann / mixed
solves, against the double oracle and the sphere's analytic solutions.

Tolerances (relative Frobenius): 1e-10 for float64 kernels, 1e-5 for float32 kernels
against the float64 oracle.  Solutions on the unit sphere (u = z) within the discretisation
error the oracle itself shows at the same level (tests/test_laplace_sym_cpu.py).
"""
import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _mesh(pkg, name, golden, dev, dt):
    if name in golden:
        v, f = golden[name]["verts"], golden[name]["faces"]
    else:
        v, f = pkg.meshes.icosphere(int(name[-1]), 1.0)
    return v, f, torch.tensor(v, dtype=dt, device=dev), torch.tensor(f, dtype=torch.int32, device=dev)


@pytest.mark.parametrize("name", ["ico1", "ell1"])
@pytest.mark.parametrize("layer", [1, 2])
@pytest.mark.parametrize("order", [0, 1])
def test_sym_panels_match_oracle(pkg, cuda, oracle, golden, name, layer, order):
    v, f, _, _ = _mesh(pkg, name, golden, cuda, torch.float64)
    ref = oracle.laplace_sym(v, f, layer, order)
    for dt, tol in ((torch.float64, 1e-10), (torch.float32, 1e-5)):
        vt = torch.tensor(v, dtype=dt, device=cuda)
        ft = torch.tensor(f, dtype=torch.int32, device=cuda)
        out = pkg.layers.laplace_sym_panels(vt, ft, layer, order)
        assert rel_err(out.cpu().numpy(), ref) < tol, (dt, layer, order)


def test_sym_panels_row_window_and_given_pairs(pkg, cuda, oracle, golden):
    v, f, vt, ft = _mesh(pkg, "ell1", golden, cuda, torch.float64)
    near = pkg.layers.laplace_near_pairs(ft)
    out = pkg.layers.laplace_sym_panels(vt, ft, 2, 1, near=near, rows=(7, 53))
    ref = oracle.laplace_sym(v, f, 2, 1, rows=(7, 53))
    assert rel_err(out.cpu().numpy(), ref) < 1e-10


def test_hypersingular_from_v0_matches_definition(pkg, cuda, oracle, golden):
    v, f, vt, ft = _mesh(pkg, "ell1", golden, cuda, torch.float64)
    v0 = oracle.laplace_sym(v, f, 1, 0)[:, :, 0, 0]
    p0, p1, p2 = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    a = 0.5 * np.linalg.norm(np.cross(p1 - p0, p2 - p1), axis=1)
    c = np.stack([p1 - p2, p2 - p0, p0 - p1], 1) / (2 * a[:, None, None])
    ref = np.einsum("yad,xbd->yxab", c, c) * v0[:, :, None, None]
    out = pkg.layers.hypersingular_from_v0(vt, ft, torch.tensor(v0, device=cuda))
    assert rel_err(out.cpu().numpy(), ref) < 1e-12
    # the reference rule's entry point (HYPERSINGULAR layer type) builds it from its own P0 V
    U = pkg.utils
    p, w1 = U.get_gaussion_integration_points_and_weights(3, device=cuda, dtype=torch.float64)
    rands, w = U.collapsed_rule_2d(p, w1)
    areas = U.compute_face_areas(vt, ft).contiguous()
    normals = U.compute_face_normals(vt, ft).contiguous()
    rel = U.compute_panel_relation(ft)
    d_ref_rule = pkg.double_integration_on_panels_3d(0, 1, vt, ft, areas, normals, w, w, rands, rands, rel, 1.0,
                                                     int(pkg.LayerType.HYPERSINGULAR_LAYER))
    v0_ref = oracle.laplace_panels(v, f, areas.cpu().numpy(), normals.cpu().numpy(), rands.cpu().numpy(),
                                   w.cpu().numpy(), rel.cpu().numpy(), 1, 0)[:, :, 0, 0]
    ref2 = np.einsum("yad,xbd->yxab", c, c) * v0_ref[:, :, None, None]
    assert rel_err(d_ref_rule.cpu().numpy(), ref2) < 1e-10
    # D annihilates constants: every packed row sums to zero
    packed = U.pack_matrix_tight(1, out, vt, ft)
    assert packed.sum(1).abs().max().item() < 1e-12 * packed.abs().max().item() * len(v)


@pytest.mark.parametrize("dt,tol", [(torch.float64, 1e-10), (torch.float32, 1e-5)])
def test_collocation_matches_oracle(pkg, cuda, oracle, golden, dt, tol):
    v, f, _, _ = _mesh(pkg, "ell1", golden, cuda, dt)
    ref = oracle.laplace_colloc_sl(v, f)
    vt = torch.tensor(v, dtype=dt, device=cuda)
    ft = torch.tensor(f, dtype=torch.int32, device=cuda)
    out = pkg.layers.laplace_colloc_sl(vt, ft)
    assert rel_err(out.cpu().numpy(), ref) < tol
    part = pkg.layers.laplace_colloc_sl(vt, ft, rows=(10, 30))
    assert rel_err(part.cpu().numpy(), ref[10:30]) < tol


def _solver(pkg, dev, dt):
    return pkg.MeshBEMSolver3d(gaussQR=3, order_type=1, BEM_type=int(pkg.BEMType.LAPLACE), wavenumber=1.0,
                               logger=None, dtype=dt, device=dev, rule="dunavant7")


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_sphere_dirichlet_neumann_mixed_solves(pkg, cuda, dt):
    v_np, f_np = pkg.meshes.icosphere(3, 1.0)
    v = torch.tensor(v_np, dtype=dt, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    z = v[:, 2:3].clone()
    nv = v.shape[0]
    solver = _solver(pkg, cuda, dt)
    D_, N_ = int(pkg.BoundaryType.DIRICHLET), int(pkg.BoundaryType.NEUMANN)
    zero = torch.zeros_like(z)
    # all Dirichlet: t = du/dn = z
    flags = torch.full((1, nv, 1), D_, dtype=torch.uint8, device=cuda)
    neu, dirv = solver.solve(v, f, z[None], zero[None], flags)
    assert (torch.linalg.norm(neu[0] - z) / torch.linalg.norm(z)).item() < 0.01
    assert torch.equal(dirv[0], z)
    # all Neumann: u = z up to a constant (zero mean of the stabilised solve)
    flags = torch.full((1, nv, 1), N_, dtype=torch.uint8, device=cuda)
    neu, dirv = solver.solve(v, f, zero[None], z[None], flags)
    u = dirv[0]
    assert (torch.linalg.norm(u - u.mean() - z) / torch.linalg.norm(z)).item() < 0.01
    # mixed: Dirichlet on the upper half, Neumann below
    flags = torch.where(z > 0, D_, N_).to(torch.uint8)[None]
    g = torch.where(z > 0, z, 0.0)[None]
    h = torch.where(z > 0, 0.0, z)[None]
    neu, dirv = solver.solve(v, f, g, h, flags)
    lower = (z <= 0).reshape(-1)
    assert (torch.linalg.norm(dirv[0][lower] - z[lower]) / torch.linalg.norm(z[lower])).item() < 0.01
    far = (z > 0.3).reshape(-1)
    assert (torch.linalg.norm(neu[0][far] - z[far]) / torch.linalg.norm(z[far])).item() < 0.05
    assert torch.equal(dirv[0][~lower], z[~lower]) and torch.equal(neu[0][lower], z[lower])


@pytest.mark.parametrize("dt,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_row_packing_and_packed_hypersingular(pkg, cuda, dt, tol):
    """mb_pack_tight_* (P1, row-accumulating path) against np.add.at, and the packed
    hypersingular matrix straight from V0 against packing the stored panels."""
    v_np, f_np = pkg.meshes.icosphere(3, 1.0)
    nf, nv = f_np.shape[0], v_np.shape[0]
    m = np.random.default_rng(3).normal(size=(nf, nf, 3, 3))
    ref = np.zeros((nv, nv))
    np.add.at(ref, (f_np[:, None, :, None], f_np[None, :, None, :]), m)
    vt = torch.tensor(v_np, dtype=dt, device=cuda)
    ft = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    got = pkg.utils.pack_matrix_tight(1, torch.tensor(m, dtype=dt, device=cuda), vt, ft)
    assert rel_err(got.cpu().numpy(), ref) < tol
    v0 = pkg.layers.laplace_sym_panels(vt, ft, 1, 0)
    d_ref = pkg.utils.pack_matrix_tight(1, pkg.layers.hypersingular_from_v0(vt, ft, v0), vt, ft)
    d_got = pkg.layers.hypersingular_tight(vt, ft, v0)
    assert rel_err(d_got.cpu().numpy(), d_ref.cpu().numpy()) < tol
    # rows sum to zero (D annihilates constants)
    assert d_got.double().sum(1).abs().max().item() < 1e3 * tol * d_got.abs().max().item()


@pytest.mark.parametrize("name", ["ico1", "ell1", "ico3"])
@pytest.mark.parametrize("dt,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_packed_operators_match_packed_panels(pkg, cuda, golden, name, dt, tol):
    """mb_laplace_sym_tight_* (no panels stored) against packing the stored panels."""
    v, f, vt, ft = _mesh(pkg, name, golden, cuda, dt)
    L, U = pkg.layers, pkg.utils
    near = L.laplace_near_pairs(ft)
    for op in (1, 2):
        ref = U.pack_matrix_tight(1, L.laplace_sym_panels(vt, ft, op, 1, near), vt, ft)
        got = L.laplace_sym_tight(vt, ft, op, near)
        assert rel_err(got.cpu().numpy(), ref.cpu().numpy()) < tol, op
    ref = L.hypersingular_tight(vt, ft, L.laplace_sym_panels(vt, ft, 1, 0, near))
    got = L.laplace_sym_tight(vt, ft, 3)
    assert rel_err(got.cpu().numpy(), ref.cpu().numpy()) < tol
    # test-row windows add up to the whole operator
    k = ft.shape[0] // 3
    part = L.laplace_sym_tight(vt, ft, 2, near, rows=(0, k))
    L.laplace_sym_tight(vt, ft, 2, near, rows=(k, ft.shape[0]), out=part)
    full = L.laplace_sym_tight(vt, ft, 2, near)
    assert rel_err(part.cpu().numpy(), full.cpu().numpy()) < tol


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_schur_solver_matches_lu(pkg, cuda, dt):
    """solver="schur" (Cholesky factors of V and of the Schur complement, symmetric parts)
    against LU of the block system: Dirichlet, Neumann and mixed data on the L3 sphere."""
    v_np, f_np = pkg.meshes.icosphere(3, 1.0)
    v = torch.tensor(v_np, dtype=dt, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    z = v[:, 2:3].clone()
    nv = v.shape[0]
    D_, N_ = int(pkg.BoundaryType.DIRICHLET), int(pkg.BoundaryType.NEUMANN)
    lu = _solver(pkg, cuda, dt)
    ch = pkg.MeshBEMSolver3d(gaussQR=3, order_type=1, BEM_type=int(pkg.BEMType.LAPLACE), wavenumber=1.0,
                             logger=None, dtype=dt, device=cuda, rule="dunavant7", solver="schur")
    zero = torch.zeros_like(z)
    cases = [(torch.full((1, nv, 1), D_, dtype=torch.uint8, device=cuda), z[None], zero[None]),
             (torch.full((1, nv, 1), N_, dtype=torch.uint8, device=cuda), zero[None], z[None]),
             (torch.where(z > 0, D_, N_).to(torch.uint8)[None], torch.where(z > 0, z, 0.0)[None],
              torch.where(z > 0, 0.0, z)[None])]
    for flags, g, h in cases:
        a = lu.solve(v, f, g, h, flags)
        b = ch.solve(v, f, g, h, flags)
        for x, y in zip(a, b):
            # the two differ by the asymmetry of the assembled operators (quadrature error)
            assert (torch.linalg.norm(x - y) / torch.linalg.norm(x)).item() < 2e-3
    # Amat_scaler scales the matrix only: the solution scales by its inverse, as with LU
    flags, g, h = cases[2]
    a = lu.solve(v, f, g, h, flags, Amat_scaler=4.0)
    b = ch.solve(v, f, g, h, flags, Amat_scaler=4.0)
    for x, y in zip(a, b):
        assert (torch.linalg.norm(x - y) / torch.linalg.norm(x)).item() < 2e-3


def test_mixed_solve_gmres_matches_lu(pkg, cuda):
    """solver="gmres" (mb_gmres_f32 on the block system) gives the LU solution."""
    v_np, f_np = pkg.meshes.icosphere(3, 1.0)
    v = torch.tensor(v_np, dtype=torch.float32, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    z = v[:, 2:3].clone()
    D_, N_ = int(pkg.BoundaryType.DIRICHLET), int(pkg.BoundaryType.NEUMANN)
    flags = torch.where(z > 0, D_, N_).to(torch.uint8)[None]
    g = torch.where(z > 0, z, 0.0)[None]
    h = torch.where(z > 0, 0.0, z)[None]
    lu = _solver(pkg, cuda, torch.float32).solve(v, f, g, h, flags)
    it = pkg.MeshBEMSolver3d(gaussQR=3, order_type=1, BEM_type=int(pkg.BEMType.LAPLACE), wavenumber=1.0,
                             logger=None, dtype=torch.float32, device=cuda, rule="dunavant7", solver="gmres",
                             gmres_tol=1e-7)
    gm = it.solve(v, f, g, h, flags)
    info = it.last_solve_info[0]
    assert info["converged"] and info["rel_residual"] < 1e-7
    for a, b in zip(lu, gm):
        assert (torch.linalg.norm(a - b) / torch.linalg.norm(a)).item() < 1e-4


@pytest.mark.parametrize("dt,tol", [(torch.float64, 0.012), (torch.float32, 0.012)])
def test_collocation_sphere_density(pkg, cuda, dt, tol):
    """V sigma = 1 on the sphere of radius a has sigma = 1/a (GMRES on the collocation matrix)."""
    a = 1.5
    v_np, f_np = pkg.meshes.icosphere(3, a)
    v = torch.tensor(v_np, dtype=dt, device=cuda)
    f = torch.tensor(f_np, dtype=torch.int32, device=cuda)
    A = pkg.layers.laplace_colloc_sl(v, f)
    ones = torch.ones(A.shape[0], dtype=torch.float64, device=cuda)
    sigma, info = pkg.mesh_MOM_3d.gmres_real(A, ones, restart=30, tol=1e-10, max_iters=500)
    assert info[0]["converged"] and info[0]["rel_residual"] < 1e-10
    assert (sigma * a - 1).abs().max().item() < tol
    lu = torch.linalg.solve(A.double(), ones)
    assert (sigma - lu).abs().max().item() < 1e-8 * lu.abs().max().item()


@pytest.mark.parametrize("n", [1000, 1003])
def test_gmres_real_matches_lu(pkg, cuda, n):
    """Real GMRES on a diagonally dominant random system (n % 4 != 0 takes the scalar path)."""
    g = torch.Generator(device="cpu").manual_seed(n)
    A64 = torch.randn(n, n, generator=g, dtype=torch.float64) / n ** 0.5 + 3 * torch.eye(n, dtype=torch.float64)
    b = torch.randn(n, generator=g, dtype=torch.float64)
    ref = torch.linalg.solve(A64, b)
    for dt in (torch.float32, torch.float64):
        A = A64.to(dt).to(cuda)
        x, info = pkg.mesh_MOM_3d.gmres_real(A, b.to(cuda), restart=20, tol=1e-12, max_iters=400)
        assert info[0]["converged"]
        exact = torch.linalg.solve(A.double().cpu(), b)  # the system actually solved
        assert (x.cpu() - exact).abs().max().item() < 1e-9 * exact.abs().max().item()
        assert (x.cpu() - ref).abs().max().item() < (1e-5 if dt == torch.float32 else 1e-10)


class _OracleBEM:
    """Mixed Laplace solve on the CPU from the oracle's symmetric-rule operators."""

    def __init__(self, ops):
        self.v, self.f, self.V, self.K, self.D, self.M = ops

    def solve(self, verts, faces, vert_bc_Dirichlet, vert_bc_Neumann, vert_bc_flags, Amat_scaler=None):
        V, K, D, M = self.V, self.K, self.D, self.M
        flags = vert_bc_flags[0].reshape(-1).cpu().numpy()
        d, n = flags == 0, flags == 1
        g = np.where(d, vert_bc_Dirichlet[0].reshape(-1).cpu().numpy(), 0.0)
        h = np.where(n, vert_bc_Neumann[0].reshape(-1).cpu().numpy(), 0.0)
        Ks = K.T
        A = np.block([[V[np.ix_(d, d)], -Ks[np.ix_(d, n)]], [Ks.T[np.ix_(n, d)], D[np.ix_(n, n)]]])
        x = np.linalg.solve(A, np.concatenate([(0.5 * M @ g + Ks @ g - V @ h)[d],
                                               (0.5 * M @ h - Ks.T @ h - D @ g)[n]]))
        neu, dirv = h.copy(), g.copy()
        neu[d], dirv[n] = x[:d.sum()], x[d.sum():]
        return torch.tensor(neu).reshape(1, -1, 1), torch.tensor(dirv).reshape(1, -1, 1)


def test_mesh_pressure_projection(pkg, cuda, oracle):
    """MeshPressure.solve on the GPU equals the same projection run on the CPU with the
    oracle's operators, and the projected velocity has no normal component on the solid
    (Neumann) vertices.  Hydrostatic data: p = rho g y on the air side, vel = (0, g dt, 0)."""
    from test_laplace_sym_cpu import _operators

    ops = _operators(pkg, oracle, 3)
    v = torch.tensor(ops[0], dtype=torch.float64, device=cuda)
    f = torch.tensor(ops[1], dtype=torch.int32, device=cuda)
    g, rho, dt = 9.8, 2.0, 0.01
    mp = pkg.MeshPressure(density_fluid=rho, gravity_strength=g, surface_tension=0.07, contact_angle=0.0,
                          gaussQR=3, order_type=1, logger=None, device=cuda, dtype=torch.float64)
    flags = torch.where(v[:, 1:2] > 0, int(pkg.BoundaryType.DIRICHLET), int(pkg.BoundaryType.NEUMANN))
    flags = flags.to(torch.uint8)[None]
    vel = torch.zeros((1, v.shape[0], 3), dtype=torch.float64, device=cuda)
    vel[..., 1] = g * dt
    new = mp.solve(v, f, dt, vel, flags)
    cpu = pkg.MeshPressure.__new__(pkg.MeshPressure)
    cpu.__dict__.update(mp.__dict__)
    cpu.gravity = mp.gravity.cpu()
    cpu.BEM_solver = _OracleBEM(ops)
    ref = cpu.solve(v.cpu(), f.cpu(), dt, vel.cpu(), flags.cpu())
    assert rel_err(new.cpu().numpy(), ref.numpy()) < 1e-7
    n = pkg.utils.compute_vert_normals(v, f)
    solid = (flags[0, :, 0] == int(pkg.BoundaryType.NEUMANN))
    vn = (new[0] * n).sum(-1)[solid].abs()
    assert vn.max().item() < 0.03 * g * dt

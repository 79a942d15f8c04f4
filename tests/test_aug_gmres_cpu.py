"""CPU checks of the algorithms behind the augmented lockstep GMRES and the compensated
refinement residual, on their numpy restatements (tests/aug_gmres_reference.py)."""
import numpy as np

from aug_gmres_reference import aug_gmres, augmentation_basis, compensated_residual


def _system(n=120, seed=0, small=0):
    rng = np.random.default_rng(seed)
    if small:  # eigenvalues in [1, 2] except `small` near 1e-3: restarted GMRES stalls on them
        lam = rng.uniform(1.0, 2.0, n) * np.exp(2j * np.pi * rng.uniform(-0.05, 0.05, n))
        lam[:small] = 1e-3 * (1 + rng.uniform(0, 1, small))
        X = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        X /= np.linalg.norm(X, axis=0)
        X = X + 3 * np.eye(n)
        Z = X @ np.diag(lam) @ np.linalg.inv(X)
        return Z, X[:, :small]
    Z = np.eye(n) * (2 + 1j) + (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) / np.sqrt(n)
    return Z, None


def test_augmented_gmres_matches_lu():
    Z, _ = _system()
    rng = np.random.default_rng(1)
    b = rng.normal(size=120) + 1j * rng.normal(size=120)
    U = rng.normal(size=(120, 8)) + 1j * rng.normal(size=(120, 8))
    Q, Ut = augmentation_basis(Z, U)
    assert np.allclose(Q.conj().T @ Q, np.eye(8), atol=1e-10)
    assert np.allclose(Z @ Ut, Q, atol=1e-10)
    M = np.diag(1.0 / np.diag(Z))  # a simple right preconditioner
    x, steps, cycles, hist = aug_gmres(Z, b, Q, Ut, M=M, restart=15, tol=1e-11)
    ref = np.linalg.solve(Z, b)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-9
    assert hist[-1] < 1e-11
    # the true residual never grows from one cycle start to the next
    assert all(b_ <= a_ * (1 + 1e-9) for a_, b_ in zip(hist, hist[1:]))


def test_subspace_holding_the_solution_needs_no_step():
    Z, _ = _system(seed=2)
    rng = np.random.default_rng(3)
    B = rng.normal(size=(120, 2)) + 1j * rng.normal(size=(120, 2))
    X = np.linalg.solve(Z, B)
    U = np.concatenate([X.real, X.imag], 1).astype(complex)
    Q, Ut = augmentation_basis(Z, U)
    for c in range(2):
        x, steps, cycles, _ = aug_gmres(Z, B[:, c], Q, Ut, restart=10, tol=1e-10)
        assert steps == 0 and cycles == 0
        assert np.linalg.norm(x - X[:, c]) / np.linalg.norm(X[:, c]) < 1e-10


def test_deflating_the_small_eigenvalues_saves_steps():
    """Eight eigenvalues near 1e-3 among the rest in [1, 2]: GMRES(12) needs many restarts;
    with their eigenvectors as the augmentation subspace it converges like the well-
    conditioned rest."""
    Z, Xs = _system(n=160, seed=4, small=8)
    rng = np.random.default_rng(5)
    b = rng.normal(size=160) + 1j * rng.normal(size=160)
    ref = np.linalg.solve(Z, b)
    x0, steps0, _, _ = aug_gmres(Z, b, restart=12, tol=1e-8, max_iters=3000)
    Q, Ut = augmentation_basis(Z, Xs)
    x1, steps1, _, _ = aug_gmres(Z, b, Q, Ut, restart=12, tol=1e-8, max_iters=3000)
    assert np.linalg.norm(x1 - ref) / np.linalg.norm(ref) < 1e-4
    assert steps1 * 2 < steps0, (steps0, steps1)


def test_dropped_directions_keep_z_ut_equal_to_q():
    """A subspace with repeated directions: the dependent ones get zero columns in both Q and
    Ut, so Z Ut = Q still holds exactly and the solve is unaffected."""
    Z, _ = _system(seed=6)
    rng = np.random.default_rng(7)
    u = rng.normal(size=(120, 1)) + 1j * rng.normal(size=(120, 1))
    U = np.concatenate([u, 2 * u, u, rng.normal(size=(120, 1)) + 0j], 1)
    Q, Ut = augmentation_basis(Z, U)
    assert np.count_nonzero(np.linalg.norm(Q, axis=0) > 1e-12) == 2
    assert np.allclose(Z @ Ut, Q, atol=1e-10)
    b = rng.normal(size=120) + 1j * rng.normal(size=120)
    x, _, _, _ = aug_gmres(Z, b, Q, Ut, restart=20, tol=1e-11)
    assert np.linalg.norm(Z @ x - b) / np.linalg.norm(b) < 1e-10


def test_compensated_residual_is_fp64_class():
    """b = Z x_true in FP64 and x = x_true + a 1e-9 perturbation: the true residual is ~1e-9 of
    |b|.  The compensated FP32 residual recovers it to a small fraction of its size; plain FP32
    sums are off by more than the residual itself."""
    rng = np.random.default_rng(8)
    n = 96
    Z = ((rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) / np.sqrt(n) + 3 * np.eye(n)).astype(np.complex64)
    Z64 = Z.astype(np.complex128)
    xt = rng.normal(size=n) + 1j * rng.normal(size=n)
    b = Z64 @ xt
    x = xt + 1e-9 * (rng.normal(size=n) + 1j * rng.normal(size=n))
    exact = b - Z64 @ x
    got = compensated_residual(Z, x, b)
    assert np.linalg.norm(got - exact) < 1e-3 * np.linalg.norm(exact)
    naive = b - (Z @ x.astype(np.complex64)).astype(np.complex128)
    assert np.linalg.norm(naive - exact) > np.linalg.norm(exact)


def test_binary16_products_with_exact_refinement_reach_fp64_accuracy():
    """Arnoldi products on a binary16 copy of Z (relative rounding ~5e-4) limit only how much
    each cycle gains; with every cycle restarted from the exact residual the iterate reaches a
    1e-10 residual, and the total products stay close to those of the exact-Z GMRES."""
    from aug_gmres_reference import half_refined_gmres

    Z, _ = _system(n=150, seed=9)
    rng = np.random.default_rng(10)
    b = rng.normal(size=150) + 1j * rng.normal(size=150)
    x, cycles, products = half_refined_gmres(Z, b, restart=40, inner_rtol=3e-3, tol=1e-10)
    ref = np.linalg.solve(Z, b)
    assert np.linalg.norm(Z @ x - b) / np.linalg.norm(b) <= 1e-10
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-9
    _, steps_exact, _, _ = aug_gmres(Z, b, restart=40, tol=1e-10)
    assert cycles >= 2 and products <= 2 * steps_exact, (cycles, products, steps_exact)

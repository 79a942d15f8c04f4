"""Numpy restatements of three solver algorithms of the GPU path (test infrastructure only).

* ``aug_gmres``: restarted right-preconditioned GMRES with a fixed augmentation subspace U
  (GCRO with a fixed recycled space), the algorithm of ``mb_gmres_blockdiag_aug_c64`` for one
  column.  With C = Z U = Q S V^H (orthonormal basis Q of Z U) and Ut = U V S^-1 (Z Ut = Q),
  a cycle starts with x += Ut Q^H r, r -= Q Q^H r; Arnoldi runs on (I - Q Q^H) Z M keeping
  b_j = Q^H Z M v_j; the cycle ends with x += M V y - Ut (B y).
* ``compensated_residual``: b - Z x by the compensated FP32 dot products of
  ``residual_c64x_kernel`` / ``bd_residual_kernel`` -- x split into FP32 hi + lo parts,
  every product Z_ij x_hi,j made exact (TwoProduct), running sums exact (TwoSum), the rounding
  terms and the x_lo products summed beside them.  Float32 arithmetic is numpy's
  round-to-nearest; the exact product error uses float64 (a product of two float32 values is
  exact in float64), which is what the GPU's fused multiply-add gives.
* ``half_refined_gmres``: GMRES cycles whose Arnoldi products read a binary16 copy of Z, each
  started from the exact residual and ended at a fixed reduction of its own estimate
  (``mb_pgmres_c64`` with ``Z_half``).
"""
from __future__ import annotations

import numpy as np


def augmentation_basis(Z: np.ndarray, U: np.ndarray, rel: float = 1e-6):
    """(Q, Ut) with Z Ut = Q, from the Gram matrix of C = Z U (directions with singular value
    below rel of the largest dropped)."""
    C = Z @ U
    lam, V = np.linalg.eigh(C.conj().T @ C)
    keep = lam > rel * rel * lam[-1]
    inv = np.where(keep, 1.0 / np.sqrt(np.maximum(lam, 1e-300)), 0.0)
    VS = V * inv[None, :]
    return C @ VS, U @ VS


def aug_gmres(Z, b, Q=None, Ut=None, M=None, restart=30, tol=1e-10, max_iters=2000):
    """x, steps, cycles, residual history (true relative residual at each cycle start)."""
    n = Z.shape[0]
    M = np.eye(n, dtype=Z.dtype) if M is None else M
    x = np.zeros(n, dtype=np.result_type(Z, b))
    bn = np.linalg.norm(b)
    steps, cycles, hist = 0, 0, []
    while True:
        r = b - Z @ x
        if Q is not None:  # cycle start: the residual-minimising combination of the subspace
            c = Q.conj().T @ r
            x = x + Ut @ c
            r = r - Q @ c
        beta = np.linalg.norm(r)
        hist.append(np.linalg.norm(b - Z @ x) / bn)
        if beta / bn <= tol or steps >= max_iters:
            return x, steps, cycles, hist
        cycles += 1
        V = np.zeros((n, restart + 1), dtype=x.dtype)
        H = np.zeros((restart + 1, restart), dtype=x.dtype)
        K = 0 if Q is None else Q.shape[1]
        B = np.zeros((K, restart), dtype=x.dtype)
        V[:, 0] = r / beta
        j_end = 0
        for j in range(restart):
            w = Z @ (M @ V[:, j])
            if Q is not None:
                B[:, j] = Q.conj().T @ w
                w = w - Q @ B[:, j]
            for _ in range(2):  # CGS2
                h = V[:, :j + 1].conj().T @ w
                H[:j + 1, j] += h
                w = w - V[:, :j + 1] @ h
            H[j + 1, j] = np.linalg.norm(w)
            j_end = j + 1
            steps += 1
            e1 = np.zeros(j + 2, dtype=x.dtype)
            e1[0] = beta
            y, *_ = np.linalg.lstsq(H[:j + 2, :j + 1], e1, rcond=None)
            res = np.linalg.norm(e1 - H[:j + 2, :j + 1] @ y)
            if res / bn <= 0.5 * tol or H[j + 1, j] == 0 or steps >= max_iters:
                break
            V[:, j + 1] = w / H[j + 1, j]
        x = x + M @ (V[:, :j_end] @ y)
        if Q is not None:
            x = x - Ut @ (B[:, :j_end] @ y)


def _two_sum(s, t):
    u = np.float32(s + t)
    bb = np.float32(u - s)
    e = np.float32(np.float32(s - np.float32(u - bb)) + np.float32(t - bb))
    return u, e


def _two_prod(a, b):
    p = np.float32(a * b)
    e = np.float32(np.float64(a) * np.float64(b) - np.float64(p))
    return p, e


def compensated_residual(Z: np.ndarray, x: np.ndarray, b: np.ndarray, lanes: int = 32) -> np.ndarray:
    """b - Z x (complex128 result) with Z complex64, x complex128, b complex128, as the GPU
    computes it: per row `lanes` interleaved partial chains (lane l takes columns l, l + lanes,
    ...), each chain compensated in FP32, the lane results added in FP64."""
    Z = Z.astype(np.complex64)
    xh = x.astype(np.complex64)
    xl = (x - xh.astype(np.complex128)).astype(np.complex64)
    n = Z.shape[0]
    r = np.zeros(n, dtype=np.complex128)
    for i in range(n):
        tot_r = 0.0
        tot_i = 0.0
        for lane in range(lanes):
            sr = si = cr = ci = np.float32(0.0)
            for j in range(lane, Z.shape[1], lanes):
                ax, ay = np.float32(Z[i, j].real), np.float32(Z[i, j].imag)
                hr, hi = np.float32(xh[j].real), np.float32(xh[j].imag)
                lr, li = np.float32(xl[j].real), np.float32(xl[j].imag)
                p1, e1 = _two_prod(ax, hr)
                p2, e2 = _two_prod(-ay, hi)
                p3, e3 = _two_prod(ax, hi)
                p4, e4 = _two_prod(ay, hr)
                sr, t1 = _two_sum(sr, p1)
                sr, t2 = _two_sum(sr, p2)
                si, t3 = _two_sum(si, p3)
                si, t4 = _two_sum(si, p4)
                lo_r = np.float32(np.float64(ax) * lr + np.float32(-ay * li))  # fma(ax, lr, -ay li)
                lo_i = np.float32(np.float64(ax) * li + np.float32(ay * lr))
                cr = np.float32(cr + np.float32(np.float32(np.float32(t1 + t2) + np.float32(e1 + e2)) + lo_r))
                ci = np.float32(ci + np.float32(np.float32(np.float32(t3 + t4) + np.float32(e3 + e4)) + lo_i))
            tot_r += float(sr) + float(cr)
            tot_i += float(si) + float(ci)
        r[i] = b[i] - complex(tot_r, tot_i)
    return r


def half_refined_gmres(Z, b, restart=40, inner_rtol=3e-3, tol=1e-10, max_cycles=200):
    """The mixed-precision scheme of ``mb_pgmres_c64`` with a binary16 copy of Z: every cycle
    starts from the exact residual r = b - Z x, runs GMRES on Zh = scale * half(Z / scale) (the
    Arnoldi products read only the rounded copy) until its residual estimate has dropped by
    inner_rtol, and adds the correction.  Returns (x, cycles, products)."""
    scale = max(np.abs(Z.real).max(), np.abs(Z.imag).max())
    Zh = (Z.real / scale).astype(np.float16).astype(np.float64) + 1j * (Z.imag / scale).astype(
        np.float16).astype(np.float64)
    Zh = Zh * scale
    x = np.zeros(Z.shape[0], dtype=complex)
    bn = np.linalg.norm(b)
    products = 0
    for cycle in range(max_cycles):
        r = b - Z @ x
        beta = np.linalg.norm(r)
        if beta / bn <= tol:
            return x, cycle, products
        n = Z.shape[0]
        V = np.zeros((n, restart + 1), dtype=complex)
        H = np.zeros((restart + 1, restart), dtype=complex)
        V[:, 0] = r / beta
        for j in range(restart):
            w = Zh @ V[:, j]
            products += 1
            for _ in range(2):
                h = V[:, :j + 1].conj().T @ w
                H[:j + 1, j] += h
                w = w - V[:, :j + 1] @ h
            H[j + 1, j] = np.linalg.norm(w)
            e1 = np.zeros(j + 2, dtype=complex)
            e1[0] = beta
            y, *_ = np.linalg.lstsq(H[:j + 2, :j + 1], e1, rcond=None)
            est = np.linalg.norm(e1 - H[:j + 2, :j + 1] @ y)
            if est <= max(inner_rtol * beta, 0.5 * tol * bn) or H[j + 1, j] == 0:
                break
            V[:, j + 1] = w / H[j + 1, j]
        x = x + V[:, :j + 1] @ y
    return x, max_cycles, products

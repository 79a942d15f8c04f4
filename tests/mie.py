"""Mie series for a perfectly conducting sphere (test infrastructure).

Time convention e^{+j w t}, free space with eps = mu = 1 (eta = 1, w = k), matching the
MoM kernels' Green's function e^{-jkR}/(4 pi R).  Incident wave E = x e^{-jkz},
H = y e^{-jkz}.

Fields come from the radial Debye potentials A_r (TM to r) and F_r (TE to r)
(R. F. Harrington, Time-Harmonic Electromagnetic Fields, 1961, ch. 6):
    E = -curl(r F_r) + (1/jk) curl curl(r A_r),   H = curl(r A_r) + (1/jk) curl curl(r F_r)
with, for the plane wave,
    A_r = C cos(phi) sum_n a_n J_n(kr) P_n^1(cos theta),
    F_r = C sin(phi) sum_n a_n J_n(kr) P_n^1(cos theta),   a_n = j^-n (2n+1) / (n(n+1)),
J_n(x) = x j_n(x) (Riccati-Bessel), P_n^1 without the Condon-Shortley phase, C = -1/k
(fixed by matching E_r = sin(theta) cos(phi) e^{-jkr cos(theta)} term by term).
The PEC sphere of radius a adds outgoing H_n(x) = x h_n^(2)(x) terms with coefficients
-a_n J_n'(ka)/H_n'(ka) (TM) and -a_n J_n(ka)/H_n(ka) (TE), which zero the tangential E.

``self_check`` verifies both statements numerically (the expansion reproduces the plane
wave; tangential E vanishes on the sphere), so nothing here rests on a remembered sign.
``surface_current(points, k, a)`` returns J = r x H_total at points on the sphere.
"""
from __future__ import annotations

import numpy as np
from scipy.special import lpmv, spherical_jn, spherical_yn


def _riccati(n, x):
    j = spherical_jn(n, x)
    jd = spherical_jn(n, x, derivative=True)
    y = spherical_yn(n, x)
    yd = spherical_yn(n, x, derivative=True)
    J, Jd = x * j, j + x * jd
    Y, Yd = x * y, y + x * yd
    return J, Jd, J - 1j * Y, Jd - 1j * Yd  # J, J', H2, H2'


def _p1(n, u):
    """P_n^1(u) without the Condon-Shortley phase and dP_n^1/du."""
    p = -lpmv(1, n, u)
    s2 = np.maximum(1.0 - u * u, 1e-300)
    # (1-u^2) dP_n^m/du = (n+m) P_{n-1}^m - n u P_n^m   (m = 1)
    pm1 = -lpmv(1, n - 1, u) if n > 1 else np.zeros_like(u)
    dp = ((n + 1) * pm1 - n * u * p) / s2
    return p, dp


def fields(points, k, a=None, n_max=None, incident=True, scattered=True):
    """E, H [N, 3] complex at Cartesian points (total, incident or scattered parts)."""
    pts = np.asarray(points, float)
    r = np.linalg.norm(pts, axis=1)
    th = np.arccos(np.clip(pts[:, 2] / r, -1, 1))
    ph = np.arctan2(pts[:, 1], pts[:, 0])
    u, st, ct = np.cos(th), np.sin(th), np.cos(th)
    kr = k * r
    if n_max is None:
        n_max = int(max(kr.max(), k * (a or 0)) + 4 * max(kr.max(), 1.0) ** (1 / 3) + 12)
    C = -1.0 / k
    Er = np.zeros(len(r), complex); Et = np.zeros_like(Er); Ep = np.zeros_like(Er)
    Hr = np.zeros_like(Er); Ht = np.zeros_like(Er); Hp = np.zeros_like(Er)
    for n in range(1, n_max + 1):
        an = (1j) ** (-n) * (2 * n + 1) / (n * (n + 1))
        J, Jd, H2, H2d = _riccati(n, kr)
        fa = np.zeros_like(Er); fad = np.zeros_like(Er)   # radial functions for A_r and F_r
        ff = np.zeros_like(Er); ffd = np.zeros_like(Er)
        if incident:
            fa += J; fad += Jd; ff += J; ffd += Jd
        if scattered:
            Ja, Jda, Ha, Hda = _riccati(n, k * a)
            ca, cf = -Jda / Hda, -Ja / Ha
            fa += ca * H2; fad += ca * H2d; ff += cf * H2; ffd += cf * H2d
        P, dP = _p1(n, u)
        dPt = -st * dP  # d/dtheta P_n^1(cos theta)
        # A_r = C an cos(phi) fa(kr) P,  F_r = C an sin(phi) ff(kr) P
        # (d_r^2 + k^2) [f(kr)] = k^2 n(n+1)/(kr)^2 f  (Riccati-Bessel equation)
        lap_a = k * k * n * (n + 1) / kr ** 2 * fa
        lap_f = k * k * n * (n + 1) / kr ** 2 * ff
        cA = C * an
        Er += (1 / (1j * k)) * cA * np.cos(ph) * lap_a * P
        Hr += (1 / (1j * k)) * cA * np.sin(ph) * lap_f * P
        # E_theta = -(1/(r sin)) dF/dphi + (1/(jk r)) d2A/(dr dtheta)
        Et += -(1 / (r * st)) * cA * np.cos(ph) * ff * P + (1 / (1j * k * r)) * cA * np.cos(ph) * k * fad * dPt
        # E_phi = (1/r) dF/dtheta + (1/(jk r sin)) d2A/(dr dphi)
        Ep += (1 / r) * cA * np.sin(ph) * ff * dPt + (1 / (1j * k * r * st)) * cA * (-np.sin(ph)) * k * fad * P
        # H_theta = (1/(r sin)) dA/dphi + (1/(jk r)) d2F/(dr dtheta)
        Ht += (1 / (r * st)) * cA * (-np.sin(ph)) * fa * P + (1 / (1j * k * r)) * cA * np.sin(ph) * k * ffd * dPt
        # H_phi = -(1/r) dA/dtheta + (1/(jk r sin)) d2F/(dr dphi)
        Hp += -(1 / r) * cA * np.cos(ph) * fa * dPt + (1 / (1j * k * r * st)) * cA * np.cos(ph) * k * ffd * P
    rh = np.stack([st * np.cos(ph), st * np.sin(ph), ct], -1)
    th_ = np.stack([ct * np.cos(ph), ct * np.sin(ph), -st], -1)
    ph_ = np.stack([-np.sin(ph), np.cos(ph), np.zeros_like(ph)], -1)
    E = Er[:, None] * rh + Et[:, None] * th_ + Ep[:, None] * ph_
    H = Hr[:, None] * rh + Ht[:, None] * th_ + Hp[:, None] * ph_
    return E, H


def surface_current(points, k, a):
    """J = r_hat x H_total on the sphere of radius a (points are projected onto it)."""
    p = np.asarray(points, float)
    p = a * p / np.linalg.norm(p, axis=1, keepdims=True)
    _, H = fields(p * (1 + 1e-12), k, a)
    rh = p / a
    return np.cross(rh, H)


def self_check(k=2.0, a=1.0, seed=0):
    """Returns (plane-wave error, tangential-E-on-surface error), both relative."""
    rng = np.random.default_rng(seed)
    pts = rng.normal(size=(200, 3))
    pts *= (0.5 + 2.5 * rng.random((200, 1))) / np.linalg.norm(pts, axis=1, keepdims=True)
    E, H = fields(pts, k, a, scattered=False)
    E0 = np.zeros_like(E); E0[:, 0] = np.exp(-1j * k * pts[:, 2])
    H0 = np.zeros_like(H); H0[:, 1] = np.exp(-1j * k * pts[:, 2])
    pw = max(np.abs(E - E0).max(), np.abs(H - H0).max())
    s = rng.normal(size=(200, 3))
    s = a * s / np.linalg.norm(s, axis=1, keepdims=True)
    Et, _ = fields(s, k, a)
    rh = s / a
    tang = Et - (Et * rh).sum(1, keepdims=True) * rh
    return pw, np.abs(tang).max()

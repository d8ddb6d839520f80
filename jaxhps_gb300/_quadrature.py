"""Spectral primitives (host side, float64 NumPy).

Same conventions as the reference's ``quadrature`` package:
Chebyshev-Lobatto points left end first (quadrature/_discretization.py:12-37),
Gauss-Legendre nodes from ``numpy.polynomial.legendre.leggauss`` (:104-116),
the Trefethen differentiation matrix (quadrature/_differentiation.py:8-47) and
barycentric Lagrange interpolation matrices (quadrature/_interpolation.py).
These run once per problem to build the small dense operators that the GPU
kernels consume; they are not on the hot path.
"""

from __future__ import annotations

import numpy as np

EPS = np.finfo(np.float64).eps


def chebyshev_points(n: int) -> np.ndarray:
    """``cos(pi*(n-1-i)/(n-1))``, i = 0..n-1 (left end first)."""
    return np.cos(np.flipud(np.pi * (np.arange(n, dtype=np.float64) / (n - 1))))


def gauss_points(n: int) -> np.ndarray:
    return np.polynomial.legendre.leggauss(n)[0]


def chebyshev_weights(n: int, bounds) -> np.ndarray:
    """Clenshaw-Curtis weights via the DCT/FFT construction of Chebfun
    (quadrature/_discretization.py:40-86)."""
    a, b = bounds
    c = 2.0 / np.concatenate([[1.0], 1.0 - np.arange(2, n, 2) ** 2])
    start = n // 2 if n % 2 else n // 2 + 1
    c = np.concatenate([c, np.flip(c[1:start])])
    w = np.fft.ifft(c).real
    out = np.concatenate([w, [w[0] / 2]])
    out[0] = w[0] / 2
    return out * (b - a) / 2


def affine_transform(pts: np.ndarray, ab) -> np.ndarray:
    a, b = ab
    return 0.5 * (b - a) * np.asarray(pts) + 0.5 * (a + b)


def differentiation_matrix_1D(points: np.ndarray) -> np.ndarray:
    x = np.asarray(points, dtype=np.float64)
    p = x.shape[0]
    c = np.where(np.arange(p) % 2 == 1, -1.0, 1.0)
    c[0] *= 2.0
    c[-1] *= 2.0
    dx = x[:, None] - x[None, :]
    d = np.outer(c, 1.0 / c) / (dx + np.eye(p))
    return d - np.diag(d.sum(axis=1))


def barycentric_lagrange_interpolation_matrix_1D(from_pts, to_pts) -> np.ndarray:
    """Rows: target points, columns: source points.  Rows whose target
    coincides with a source point are unit rows."""
    f = np.asarray(from_pts, dtype=np.float64)
    t = np.asarray(to_pts, dtype=np.float64)
    diff = f[:, None] - f[None, :]
    np.fill_diagonal(diff, 1.0)
    w = np.prod(diff, axis=0)
    dist = t[:, None] - f[None, :]
    hit = dist == 0
    with np.errstate(divide="ignore", invalid="ignore"):
        terms = 1.0 / (w[None, :] * dist)
        m = terms / terms.sum(axis=1, keepdims=True)
    rows = hit.any(axis=1)
    m[rows] = hit[rows].astype(np.float64)
    return m


def _bary_weights(x):
    diff = x[:, None] - x[None, :]
    np.fill_diagonal(diff, 1.0)
    return np.prod(diff, axis=0)


def barycentric_lagrange_interpolation_matrix_2D(from_x, from_y, to_x, to_y) -> np.ndarray:
    """Tensor-product interpolation on meshgrid(..., indexing='ij') grids,
    with coincident points nudged by EPS as in quadrature/_interpolation.py:117-213."""
    mats = []
    for f, t in ((from_x, to_x), (from_y, to_y)):
        f = np.asarray(f, dtype=np.float64)
        t = np.asarray(t, dtype=np.float64)
        w = _bary_weights(f)
        dist = t[None, :] - f[:, None]
        dist = np.where(dist == 0, EPS, dist)
        nf = np.sum(1.0 / (w[:, None] * dist), axis=0)
        mats.append(1.0 / (dist.T * w[None, :] * nf[:, None]))
    return np.kron(mats[0], mats[1])


def barycentric_lagrange_interpolation_matrix_3D(from_x, from_y, from_z, to_x, to_y, to_z) -> np.ndarray:
    mats = []
    for f, t in ((from_x, to_x), (from_y, to_y), (from_z, to_z)):
        f = np.asarray(f, dtype=np.float64)
        t = np.asarray(t, dtype=np.float64)
        w = _bary_weights(f)
        dist = t[None, :] - f[:, None]
        dist = np.where(dist == 0, EPS, dist)
        nf = np.sum(1.0 / (w[:, None] * dist), axis=0)
        mats.append(1.0 / (dist.T * w[None, :] * nf[:, None]))
    return np.kron(np.kron(mats[0], mats[1]), mats[2])

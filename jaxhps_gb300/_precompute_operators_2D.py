"""Small dense 2D operators (host side, float64), following
src/jaxhps/_precompute_operators_2D.py.  Built once per problem and copied
to the device; the GPU stages only consume them.
"""

from __future__ import annotations

import numpy as np

from ._grid_creation_2D import rearrange_indices_ext_int
from ._quadrature import (
    affine_transform,
    barycentric_lagrange_interpolation_matrix_1D,
    barycentric_lagrange_interpolation_matrix_2D,
    chebyshev_points,
    differentiation_matrix_1D,
    gauss_points,
)


def precompute_diff_operators_2D(p: int, half_side_len: float):
    """D_x, D_y, D_xx, D_yy, D_xy on the exterior-first leaf grid (:16-44)."""
    r = rearrange_indices_ext_int(p)
    d = differentiation_matrix_1D(chebyshev_points(p)) / half_side_len
    dx = np.kron(d, np.eye(p))[np.ix_(r, r)]
    dy = -np.kron(np.eye(p), d)[np.ix_(r, r)]
    return dx, dy, dx @ dx, dy @ dy, dx @ dy


def precompute_P_2D_DtN(p: int, q: int) -> np.ndarray:
    """(4(p-1), 4q) Gauss -> Chebyshev boundary map, corners averaged (:48-79)."""
    P = barycentric_lagrange_interpolation_matrix_1D(gauss_points(q), chebyshev_points(p))
    out = np.zeros((4 * (p - 1), 4 * q))
    for s in range(3):
        out[s * (p - 1):s * (p - 1) + p, s * q:(s + 1) * q] = P
    out[3 * (p - 1):, 3 * q:] = P[:-1]
    out[0, 3 * q:] = P[-1]
    out[[0, p - 1, 2 * (p - 1), 3 * (p - 1)]] *= 0.5
    return out


def precompute_P_2D_ItI(p: int, q: int) -> np.ndarray:
    """kron(I_4, P[:-1]) (:83-99)."""
    P = barycentric_lagrange_interpolation_matrix_1D(gauss_points(q), chebyshev_points(p))
    return np.kron(np.eye(4), P[:-1])


def precompute_N_matrix_2D(du_dx: np.ndarray, du_dy: np.ndarray, p: int) -> np.ndarray:
    """(4p, p^2) outward normal derivative with doubled corners (:132-163)."""
    N = np.zeros((4 * p, p * p))
    N[:p] = -du_dy[:p]
    N[p:2 * p] = du_dx[p - 1:2 * p - 1]
    N[2 * p:3 * p] = du_dy[2 * p - 2:3 * p - 2]
    N[3 * p:4 * p - 1] = -du_dx[3 * p - 3:4 * p - 4]
    N[4 * p - 1] = -du_dx[0]
    return N


def precompute_N_tilde_matrix_2D(du_dx: np.ndarray, du_dy: np.ndarray, p: int) -> np.ndarray:
    """(4(p-1), p^2) outward normal derivative at the boundary points (:166-192)."""
    m = p - 1
    N = np.zeros((4 * m, p * p))
    N[:m] = -du_dy[:m]
    N[m:2 * m] = du_dx[m:2 * m]
    N[2 * m:3 * m] = du_dy[2 * m:3 * m]
    N[3 * m:] = -du_dx[3 * m:4 * m]
    return N


def _cheby_to_gauss_sides(p: int, q: int) -> np.ndarray:
    Qi = barycentric_lagrange_interpolation_matrix_1D(chebyshev_points(p), gauss_points(q))
    return np.kron(np.eye(4), Qi)


def precompute_Q_2D_DtN(p: int, q: int, du_dx: np.ndarray, du_dy: np.ndarray) -> np.ndarray:
    """(4q, p^2) map from leaf values to outward normal derivative at Gauss nodes (:102-129)."""
    return _cheby_to_gauss_sides(p, q) @ precompute_N_matrix_2D(du_dx, du_dy, p)


def precompute_QH_2D_ItI(N: np.ndarray, p: int, q: int, eta: float) -> np.ndarray:
    """(4q, p^2) outgoing impedance u_n - i eta u at Gauss nodes (:195-240)."""
    H = N.astype(np.complex128)
    idx_rows = np.concatenate([np.arange(0, p), np.arange(p, 2 * p), np.arange(2 * p, 3 * p),
                               np.arange(3 * p, 4 * p - 1), [4 * p - 1]])
    idx_cols = np.concatenate([np.arange(0, p), np.arange(p - 1, 2 * p - 1), np.arange(2 * p - 2, 3 * p - 2),
                               np.arange(3 * p - 3, 4 * p - 4), [0]])
    H[idx_rows, idx_cols] -= 1j * eta
    return _cheby_to_gauss_sides(p, q) @ H


def precompute_G_2D_ItI(N_tilde: np.ndarray, eta: float) -> np.ndarray:
    """(4(p-1), p^2) incoming impedance u_n + i eta u at the boundary points (:243-265)."""
    G = N_tilde.astype(np.complex128)
    m = G.shape[0]
    G[np.arange(m), np.arange(m)] += 1j * eta
    return G


def precompute_projection_ops_2D(q: int):
    """Refining (2q, q) and coarsening (q, 2q) Gauss-panel maps (:268-300)."""
    g = gauss_points(q)
    refined = np.concatenate([affine_transform(g, (-1.0, 0.0)), affine_transform(g, (0.0, 1.0))])
    return (barycentric_lagrange_interpolation_matrix_1D(g, refined),
            barycentric_lagrange_interpolation_matrix_1D(refined, g))


def indexing_for_refinement_operator(p: int):
    """Row/column orderings of the 4-child refinement operator (:331-379)."""
    col = rearrange_indices_ext_int(p)
    ii = np.arange(4 * p * p)
    xh = ii % (2 * p) >= p
    yh = (ii // (2 * p)) % (2 * p) >= p
    blocks = [ii[xh & ~yh], ii[xh & yh], ii[~xh & yh], ii[~xh & ~yh]]
    return np.concatenate([b[col] for b in blocks]), col


def precompute_L_4f1(p: int) -> np.ndarray:
    """(4p^2, p^2) interpolation from a leaf grid to its four children (:303-328)."""
    c = chebyshev_points(p)
    refined = np.concatenate([affine_transform(c, (-1, 0)), affine_transform(c, (0, 1))])
    I = barycentric_lagrange_interpolation_matrix_2D(c, c, refined, refined)
    r, col = indexing_for_refinement_operator(p)
    return I[r][:, col]

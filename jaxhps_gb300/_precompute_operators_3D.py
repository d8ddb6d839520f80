"""Small dense 3D operators (host side, float64), following
src/jaxhps/_precompute_operators_3D.py.  Built once per problem and copied
to the device; the GPU stages only consume them.

Face numbering (1..6 in the reference, 0..5 here): -x, +x, -y, +y, -z, +z.
"""

from __future__ import annotations

import numpy as np

from ._grid_creation_3D import rearrange_indices_ext_int
from ._quadrature import (
    affine_transform,
    barycentric_lagrange_interpolation_matrix_1D,
    barycentric_lagrange_interpolation_matrix_2D,
    barycentric_lagrange_interpolation_matrix_3D,
    chebyshev_points,
    differentiation_matrix_1D,
    gauss_points,
)


def precompute_diff_operators_3D(p: int, half_side_len: float):
    """D_x, D_y, D_z, D_xx, D_yy, D_zz, D_xy, D_xz, D_yz on the
    exterior-first leaf grid (:17-61)."""
    r = rearrange_indices_ext_int(p)
    d = differentiation_matrix_1D(chebyshev_points(p)) / half_side_len
    I = np.eye(p)
    dx = np.kron(d, np.kron(I, I))[np.ix_(r, r)]
    dy = np.kron(I, np.kron(d, I))[np.ix_(r, r)]
    dz = np.kron(I, np.kron(I, d))[np.ix_(r, r)]
    return dx, dy, dz, dx @ dx, dy @ dy, dz @ dz, dx @ dy, dx @ dz, dy @ dz


def face_idxes(p: int, face: int) -> np.ndarray:
    """Positions (in the exterior-first order) of the p^2 Chebyshev points
    of ``face``, in raster order of the face's two tangential coordinates
    (the reference spells these out as get_face_1_idxes..get_face_6_idxes,
    :220-320)."""
    r = rearrange_indices_ext_int(p)
    pos = np.empty(p ** 3, dtype=np.int64)
    pos[r] = np.arange(p ** 3)
    idx = np.arange(p ** 3)
    coord = (idx // (p * p), (idx // p) % p, idx % p)[face // 2]
    on = coord == (0 if face % 2 == 0 else p - 1)
    return pos[idx[on]]   # idx is raster order, so the face keeps raster order


def precompute_P_3D_DtN(p: int, q: int) -> np.ndarray:
    """(p^3 - (p-2)^3, 6q^2) Gauss -> Chebyshev boundary map; points on
    several faces (edges, corners) average the faces' values (:64-147)."""
    g, c = gauss_points(q), chebyshev_points(p)
    B = barycentric_lagrange_interpolation_matrix_2D(g, g, c, c)
    n_cb = p ** 3 - (p - 2) ** 3
    P = np.zeros((n_cb, 6 * q * q))
    count = np.zeros(n_cb)
    for f in range(6):
        rows = face_idxes(p, f)
        P[rows, f * q * q:(f + 1) * q * q] = B
        count[rows] += 1
    return P / count[:, None]


def precompute_N_matrix_3D(du_dx: np.ndarray, du_dy: np.ndarray, du_dz: np.ndarray, p: int) -> np.ndarray:
    """(6p^2, p^3) outward normal derivative on each face's Chebyshev
    points (edge and corner points appear once per face)."""
    ops = (du_dx, du_dy, du_dz)
    return np.concatenate([(1.0 if f % 2 else -1.0) * ops[f // 2][face_idxes(p, f)] for f in range(6)])


def precompute_Q_3D_DtN(p: int, q: int, du_dx: np.ndarray, du_dy: np.ndarray, du_dz: np.ndarray) -> np.ndarray:
    """(6q^2, p^3) map from leaf values to the outward normal derivative at
    the boundary Gauss nodes (:150-210)."""
    g, c = gauss_points(q), chebyshev_points(p)
    B = barycentric_lagrange_interpolation_matrix_2D(c, c, g, g)
    N = precompute_N_matrix_3D(du_dx, du_dy, du_dz, p)
    return np.kron(np.eye(6), B) @ N


def precompute_projection_ops_3D(q: int):
    """Refining (4q^2, q^2) and coarsening (q^2, 4q^2) maps between one Gauss
    face panel and its four quarter panels in 2D quad order (:323-409)."""
    if q % 2:
        raise ValueError("q must be even.")
    g = gauss_points(q)
    lo, hi = affine_transform(g, (-1.0, 0.0)), affine_transform(g, (0.0, 1.0))
    quarters = ((lo, lo), (hi, lo), (hi, hi), (lo, hi))
    L_4f1 = np.concatenate([barycentric_lagrange_interpolation_matrix_2D(g, g, u, v) for u, v in quarters])
    L_1f4 = np.zeros((q * q, 4 * q * q))
    for k, (u, v) in enumerate(quarters):
        # each coarse Gauss node lies in exactly one quarter; interpolate from that quarter
        uq = (g < 0) if u is lo else (g >= 0)
        vq = (g < 0) if v is lo else (g >= 0)
        rows = (uq[:, None] & vq[None, :]).ravel()
        Bq = barycentric_lagrange_interpolation_matrix_2D(u, v, g, g)
        L_1f4[rows, k * q * q:(k + 1) * q * q] = Bq[rows]
    return L_4f1, L_1f4


def precompute_L_8f1(p: int) -> np.ndarray:
    """(8p^3, p^3) interpolation from a leaf's Chebyshev grid to the grids of
    its eight children a..h, each in exterior-first order (:412-443)."""
    c = chebyshev_points(p)
    lo, hi = affine_transform(c, (-1.0, 0.0)), affine_transform(c, (0.0, 1.0))
    r = rearrange_indices_ext_int(p)
    kids = ((lo, lo, hi), (hi, lo, hi), (hi, hi, hi), (lo, hi, hi), (lo, lo, lo), (hi, lo, lo), (hi, hi, lo),
            (lo, hi, lo))
    blocks = [barycentric_lagrange_interpolation_matrix_3D(c, c, c, x, y, z)[r][:, r] for x, y, z in kids]
    return np.concatenate(blocks)

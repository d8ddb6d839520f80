"""2D HPS grids (host side) following src/jaxhps/_grid_creation_2D.py.

Leaf order for uniform trees: repeated SW, SE, NE, NW subdivision
(:18-46).  Leaf points: meshgrid(x, flipud(y), 'ij') permuted exterior
first, counter-clockwise from the SW corner (:49-68, :203-233).  Root
boundary Gauss points: S (x up), E (y up), N (x down), W (y down) (:76-124).
"""

from __future__ import annotations

import numpy as np

from ._discretization_tree import DiscretizationNode2D, get_all_leaves
from ._quadrature import affine_transform, chebyshev_points, gauss_points


def rearrange_indices_ext_int(n: int) -> np.ndarray:
    """Flat meshgrid index (ix*n + iy, iy = 0 the north row) of every point
    in exterior-first order."""
    ix = np.arange(n)
    south = ix * n + (n - 1)
    east = (n - 1) * n + np.arange(n - 2, -1, -1)
    north = np.arange(n - 2, -1, -1) * n
    west = np.arange(1, n - 1)
    bdry = np.concatenate([south, east, north, west])
    mask = np.ones(n * n, dtype=bool)
    mask[bdry] = False
    return np.concatenate([bdry, np.nonzero(mask)[0]]).astype(np.int64)


def bounds_for_quad_subdivision(b) -> np.ndarray:
    xmin, xmax, ymin, ymax = b
    xm, ym = (xmin + xmax) / 2, (ymin + ymax) / 2
    return np.array([[xmin, xm, ymin, ym], [xm, xmax, ymin, ym], [xm, xmax, ym, ymax], [xmin, xm, ym, ymax]])


def uniform_leaf_bounds_2D(root_bounds, L: int) -> np.ndarray:
    b = np.asarray([root_bounds], dtype=np.float64)
    for _ in range(L):
        xmin, xmax, ymin, ymax = b[:, 0], b[:, 1], b[:, 2], b[:, 3]
        xm, ym = (xmin + xmax) / 2, (ymin + ymax) / 2
        kids = np.stack([
            np.stack([xmin, xm, ymin, ym], -1),
            np.stack([xm, xmax, ymin, ym], -1),
            np.stack([xm, xmax, ym, ymax], -1),
            np.stack([xmin, xm, ym, ymax], -1),
        ], axis=1)
        b = kids.reshape(-1, 4)
    return b


def bounds_to_cheby_points_2D(bounds: np.ndarray, p: int) -> np.ndarray:
    """(n_leaves, 4) bounds -> (n_leaves, p^2, 2) points, exterior first."""
    c = chebyshev_points(p)
    r = rearrange_indices_ext_int(p)
    b = np.atleast_2d(bounds)
    xs = 0.5 * (b[:, 1:2] - b[:, 0:1]) * c[None, :] + 0.5 * (b[:, 0:1] + b[:, 1:2])
    ys = 0.5 * (b[:, 3:4] - b[:, 2:3]) * c[None, :] + 0.5 * (b[:, 2:3] + b[:, 3:4])
    ys = ys[:, ::-1]
    X = np.repeat(xs[:, :, None], p, axis=2)
    Y = np.repeat(ys[:, None, :], p, axis=1)
    pts = np.stack([X.reshape(len(b), -1), Y.reshape(len(b), -1)], axis=-1)
    return pts[:, r]


def compute_interior_Chebyshev_points_uniform_2D(root: DiscretizationNode2D, L: int, p: int) -> np.ndarray:
    return bounds_to_cheby_points_2D(uniform_leaf_bounds_2D(root.bounds, L), p)


def compute_interior_Chebyshev_points_adaptive_2D(root: DiscretizationNode2D, p: int) -> np.ndarray:
    b = np.array([leaf.bounds for leaf in get_all_leaves(root)])
    return bounds_to_cheby_points_2D(b, p)


def compute_boundary_Gauss_points_uniform_2D(root: DiscretizationNode2D, L: int, q: int) -> np.ndarray:
    g = gauss_points(q)
    n = 2 ** L
    xb = np.linspace(root.xmin, root.xmax, n + 1)
    yb = np.linspace(root.ymin, root.ymax, n + 1)
    xg = np.concatenate([affine_transform(g, xb[i:i + 2]) for i in range(n)])
    yg = np.concatenate([affine_transform(g, yb[i:i + 2]) for i in range(n)])
    return np.concatenate([
        np.stack([xg, np.full_like(xg, root.ymin)], -1),
        np.stack([np.full_like(yg, root.xmax), yg], -1),
        np.stack([xg[::-1], np.full_like(xg, root.ymax)], -1),
        np.stack([np.full_like(yg, root.xmin), yg[::-1]], -1),
    ])


def compute_boundary_Gauss_points_adaptive_2D(root: DiscretizationNode2D, q: int) -> np.ndarray:
    """Root boundary Gauss points of an adaptive quadtree: q per boundary
    leaf, S (W->E), E (S->N), N (E->W), W (N->S) (:142-203)."""
    from ._discretization_tree_operations_2D import get_ordered_lst_of_boundary_nodes

    g = gauss_points(q)
    s, e, n, w = get_ordered_lst_of_boundary_nodes(root)
    xs = np.concatenate([affine_transform(g, (lf.xmin, lf.xmax)) for lf in s])
    ye = np.concatenate([affine_transform(g, (lf.ymin, lf.ymax)) for lf in e])
    xn = np.concatenate([affine_transform(g, (lf.xmax, lf.xmin)) for lf in n])
    yw = np.concatenate([affine_transform(g, (lf.ymax, lf.ymin)) for lf in w])
    return np.concatenate([
        np.stack([xs, np.full_like(xs, root.ymin)], -1),
        np.stack([np.full_like(ye, root.xmax), ye], -1),
        np.stack([xn, np.full_like(xn, root.ymax)], -1),
        np.stack([np.full_like(yw, root.xmin), yw], -1),
    ])


def get_all_uniform_leaves_2D(root: DiscretizationNode2D, L: int):
    b = uniform_leaf_bounds_2D(root.bounds, L)
    return [DiscretizationNode2D(*x, depth=L) for x in b]

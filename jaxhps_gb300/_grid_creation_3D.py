"""3D HPS grids (host side) following src/jaxhps/_grid_creation_3D.py.

Children of an octree node are a..h (:28-74): a-d in the upper z half,
e-h in the lower, each half ordered (x lo, y lo), (x hi, y lo), (x hi, y hi),
(x lo, y hi).  Leaf points: meshgrid(x, y, z, 'ij') permuted exterior first
(:420-458): the x = min face, the x = max face, then y = min / y = max
(without the x faces), then z = min / z = max (without the x and y faces),
then the interior; inside each face the tangential coordinates run in raster
order (x before y before z).  Boundary Gauss points (:119-236): faces
-x, +x, -y, +y, -z, +z; on each face the panels follow the 2D quad order
(SW, SE, NE, NW) of the face's two coordinates, and inside a panel the Gauss
points are meshgrid(..., 'ij').
"""

from __future__ import annotations

import numpy as np

from ._discretization_tree import DiscretizationNode3D, get_all_leaves
from ._grid_creation_2D import uniform_leaf_bounds_2D
from ._quadrature import affine_transform, chebyshev_points, gauss_points

# Child traversal orders that list a face's leaves in 2D quad order
# (_grid_creation_3D.py get_ordered_lst_of_boundary_nodes): faces -x/+x in
# (y, z), faces -y/+y in (x, z), faces -z/+z in (x, y).
FACE_TRAVERSAL = ((4, 7, 3, 0, 5, 6, 2, 1), (4, 5, 1, 0, 7, 6, 2, 3), (0, 1, 2, 3, 4, 5, 6, 7))


def rearrange_indices_ext_int(p: int) -> np.ndarray:
    """Raster index (ix*p^2 + iy*p + iz) of every leaf point in
    exterior-first order."""
    idx = np.arange(p ** 3)
    ix, iy, iz = idx // (p * p), (idx // p) % p, idx % p
    xf = (ix == 0) | (ix == p - 1)
    yf = ((iy == 0) | (iy == p - 1)) & ~xf
    zf = ((iz == 0) | (iz == p - 1)) & ~xf & ~yf
    groups = [ix == 0, ix == p - 1, yf & (iy == 0), yf & (iy == p - 1), zf & (iz == 0), zf & (iz == p - 1),
              ~(xf | yf | zf)]
    return np.concatenate([idx[g] for g in groups]).astype(np.int64)


def bounds_for_oct_subdivision(b) -> np.ndarray:
    """(6,) bounds -> (8, 6) bounds of the children a..h."""
    xmin, xmax, ymin, ymax, zmin, zmax = b
    xm, ym, zm = (xmin + xmax) / 2, (ymin + ymax) / 2, (zmin + zmax) / 2
    quad = [(xmin, xm, ymin, ym), (xm, xmax, ymin, ym), (xm, xmax, ym, ymax), (xmin, xm, ym, ymax)]
    return np.array([q + (zm, zmax) for q in quad] + [q + (zmin, zm) for q in quad])


def uniform_leaf_bounds_3D(root_bounds, L: int) -> np.ndarray:
    """(8^L, 6) leaf bounds; the children of node i are rows 8i..8i+7."""
    b = np.asarray([root_bounds], dtype=np.float64)
    for _ in range(L):
        b = np.concatenate([bounds_for_oct_subdivision(x) for x in b])
    return b


def bounds_to_cheby_points_3D(bounds: np.ndarray, p: int) -> np.ndarray:
    """(n_leaves, 6) bounds -> (n_leaves, p^3, 3) points, exterior first."""
    c = chebyshev_points(p)
    r = rearrange_indices_ext_int(p)
    b = np.atleast_2d(np.asarray(bounds, dtype=np.float64))
    out = np.empty((len(b), p ** 3, 3))
    for k, bb in enumerate(b):
        xs = affine_transform(c, bb[0:2])
        ys = affine_transform(c, bb[2:4])
        zs = affine_transform(c, bb[4:6])
        X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
        out[k] = np.stack([X.ravel(), Y.ravel(), Z.ravel()], -1)[r]
    return out


def compute_interior_Chebyshev_points_uniform_3D(root: DiscretizationNode3D, L: int, p: int) -> np.ndarray:
    return bounds_to_cheby_points_3D(uniform_leaf_bounds_3D(root.bounds, L), p)


def compute_interior_Chebyshev_points_adaptive_3D(root: DiscretizationNode3D, p: int) -> np.ndarray:
    return bounds_to_cheby_points_3D(np.array([leaf.bounds for leaf in get_all_leaves(root)]), p)


def _gauss_faces(face_bounds: np.ndarray, q: int) -> np.ndarray:
    """(n, 4) panel bounds (u0, u1, v0, v1) -> (n*q^2, 2) Gauss points,
    meshgrid(u, v, 'ij') inside each panel."""
    g = gauss_points(q)
    out = []
    for u0, u1, v0, v1 in np.atleast_2d(face_bounds):
        U, V = np.meshgrid(affine_transform(g, (u0, u1)), affine_transform(g, (v0, v1)), indexing="ij")
        out.append(np.stack([U.ravel(), V.ravel()], -1))
    return np.concatenate(out)


def _assemble_faces(root, panels, q: int) -> np.ndarray:
    """panels[f] = (n_f, 4) panel bounds of face f in its two tangential coordinates."""
    fixed = (root.xmin, root.xmax, root.ymin, root.ymax, root.zmin, root.zmax)
    tang = ((1, 2), (1, 2), (0, 2), (0, 2), (0, 1), (0, 1))
    out = []
    for f in range(6):
        uv = _gauss_faces(panels[f], q)
        pts = np.empty((uv.shape[0], 3))
        pts[:, f // 2] = fixed[f]
        pts[:, tang[f][0]] = uv[:, 0]
        pts[:, tang[f][1]] = uv[:, 1]
        out.append(pts)
    return np.concatenate(out)


def compute_boundary_Gauss_points_uniform_3D(root: DiscretizationNode3D, L: int, q: int) -> np.ndarray:
    """(6 q^2 4^L, 3) root boundary Gauss points (:119-236)."""
    yz = uniform_leaf_bounds_2D((root.ymin, root.ymax, root.zmin, root.zmax), L)
    xz = uniform_leaf_bounds_2D((root.xmin, root.xmax, root.zmin, root.zmax), L)
    xy = uniform_leaf_bounds_2D((root.xmin, root.xmax, root.ymin, root.ymax), L)
    return _assemble_faces(root, (yz, yz, xz, xz, xy, xy), q)


def get_all_leaves_special_ordering_3D(node, child_traversal_order=None):
    """Leaves in depth-first order, visiting children in the given order
    (_discretization_tree_operations_3D.py:7-23)."""
    order = tuple(range(8)) if child_traversal_order is None else tuple(int(c) for c in child_traversal_order)
    if not len(node.children):
        return (node,)
    out = ()
    for c in order:
        out += get_all_leaves_special_ordering_3D(node.children[c], order)
    return out


def get_ordered_lst_of_boundary_nodes(root: DiscretizationNode3D):
    """The leaves touching each of the six faces, in 2D quad order of the face."""
    out = []
    for f in range(6):
        leaves = get_all_leaves_special_ordering_3D(root, FACE_TRAVERSAL[f // 2])
        axis, hi = f // 2, f % 2
        key = ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")[2 * axis + hi]
        out.append(tuple(lf for lf in leaves if getattr(lf, key) == getattr(root, key)))
    return tuple(out)


def compute_boundary_Gauss_points_adaptive_3D(root: DiscretizationNode3D, q: int) -> np.ndarray:
    faces = get_ordered_lst_of_boundary_nodes(root)
    tang = ((1, 2), (1, 2), (0, 2), (0, 2), (0, 1), (0, 1))
    panels = []
    for f in range(6):
        a, b = tang[f]
        panels.append(np.array([(lf.bounds[2 * a], lf.bounds[2 * a + 1], lf.bounds[2 * b], lf.bounds[2 * b + 1])
                                for lf in faces[f]]))
    return _assemble_faces(root, panels, q)


def get_all_uniform_leaves_3D(root: DiscretizationNode3D, L: int):
    return [DiscretizationNode3D(*b, depth=L) for b in uniform_leaf_bounds_3D(root.bounds, L)]


def leaf_boundary_gauss_points_3D(bounds: np.ndarray, q: int) -> np.ndarray:
    """(n_leaves, 6q^2, 3) Gauss nodes of every leaf boundary, in the leaf's
    own face order (-x, +x, -y, +y, -z, +z; meshgrid 'ij' inside a face)."""
    g = gauss_points(q)
    b = np.atleast_2d(np.asarray(bounds, dtype=np.float64))
    out = np.empty((len(b), 6 * q * q, 3))
    tang = ((1, 2), (1, 2), (0, 2), (0, 2), (0, 1), (0, 1))
    for f in range(6):
        ax, side = f // 2, f % 2
        ta, tb = tang[f]
        U = 0.5 * (b[:, 2 * ta + 1:2 * ta + 2] - b[:, 2 * ta:2 * ta + 1]) * g[None] + \
            0.5 * (b[:, 2 * ta:2 * ta + 1] + b[:, 2 * ta + 1:2 * ta + 2])
        V = 0.5 * (b[:, 2 * tb + 1:2 * tb + 2] - b[:, 2 * tb:2 * tb + 1]) * g[None] + \
            0.5 * (b[:, 2 * tb:2 * tb + 1] + b[:, 2 * tb + 1:2 * tb + 2])
        sl = slice(f * q * q, (f + 1) * q * q)
        out[:, sl, ax] = b[:, 2 * ax + side][:, None]
        out[:, sl, ta] = np.repeat(U, q, axis=1)
        out[:, sl, tb] = np.tile(V, (1, q))
    return out

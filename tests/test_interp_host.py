"""Interpolation between the HPS grid and rectangular grids, host side: the
oracle pinned by the reference's polynomial known-answer cases
(tests/test_interpolation_methods.py, tests/test_domain.py), and the host
helpers of jaxhps_gb300._interpolation (leaf location through the cell table,
barycentric weights)."""

import numpy as np
import pytest

from oracle import hps_oracle as O
from jaxhps_gb300._grid_creation_2D import bounds_to_cheby_points_2D, uniform_leaf_bounds_2D
from jaxhps_gb300._grid_creation_3D import bounds_to_cheby_points_3D, uniform_leaf_bounds_3D
from jaxhps_gb300 import _interpolation as ip


def adaptive_bounds_2D():
    """[-1,1]^2 split once, its SW quarter split again, in leaf (DFS) order."""
    top = uniform_leaf_bounds_2D((-1.0, 1.0, -1.0, 1.0), 1)
    sw = uniform_leaf_bounds_2D(tuple(top[0]), 1)
    return np.concatenate([sw, top[1:]])


@pytest.mark.parametrize("bounds", [uniform_leaf_bounds_2D((-1.0, 1.0, -1.0, 1.0), 2), adaptive_bounds_2D()])
def test_oracle_interp_from_hps_2D_exact_for_quadratics(bounds):
    p = 6
    pts = bounds_to_cheby_points_2D(bounds, p)
    f = lambda x: 3 * x[..., 1] - 4 * x[..., 0] ** 2   # noqa: E731
    xv, yv = np.linspace(-1, 1, 3), np.linspace(-1, 1, 3)
    vals, tp = O.oracle_interp_from_hps(bounds, p, f(pts), [xv, yv])
    X, Y = np.meshgrid(xv, yv)
    assert np.allclose(tp[..., 0], X) and np.allclose(tp[..., 1], Y)
    assert vals.shape == (3, 3)
    assert np.allclose(vals, f(tp), atol=1e-12)


def test_oracle_interp_to_hps_2D_exact_for_quadratics():
    p, n_x, n_y = 6, 10, 11
    b = uniform_leaf_bounds_2D((-1.0, 1.0, -1.0, 1.0), 2)
    xs, ys = np.linspace(-1, 1, n_x), np.linspace(-1, 1, n_y)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    g = lambda x, y: x ** 2 - 3 * y   # noqa: E731
    out = O.oracle_interp_to_hps(b, g(X, Y), p, [xs, ys])
    pts = bounds_to_cheby_points_2D(b, p)
    assert out.shape == (16, 36)
    assert np.allclose(out, g(pts[..., 0], pts[..., 1]), atol=1e-12)


def test_oracle_interp_3D_exact_for_quadratics():
    p = 5
    b = uniform_leaf_bounds_3D((-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), 1)
    pts = bounds_to_cheby_points_3D(b, p)
    f = lambda x: x[..., 0] ** 2 - x[..., 1] * x[..., 2] + 2   # noqa: E731
    ax = [np.linspace(-1, 1, 3), np.linspace(-1, 1, 4), np.linspace(-1, 1, 2)]
    vals, tp = O.oracle_interp_from_hps(b, p, f(pts), ax)
    assert vals.shape == (3, 4, 2) and tp.shape == (4, 3, 2, 3)
    assert np.allclose(vals.reshape(-1), f(tp).reshape(-1), atol=1e-12)
    ax = [np.linspace(-1, 1, 6), np.linspace(-1, 1, 7), np.linspace(-1, 1, 5)]
    X = np.stack(np.meshgrid(*ax, indexing="ij"), -1)
    out = O.oracle_interp_to_hps(b, f(X), p, ax)
    assert np.allclose(out, f(pts), atol=1e-12)


def _locate_like_kernel(pts, bounds, cells, nc, lo, h):
    """The device kernel's leaf search restated: the floor cell, its 3^d
    neighbourhood, the smallest leaf index whose closed box holds the point."""
    d = pts.shape[1]
    out = np.zeros(len(pts), dtype=np.int64)
    for k, x in enumerate(pts):
        base = [int(min(max(np.floor((x[a] - lo[a]) / h[a]), 0), nc[a] - 1)) for a in range(d)]
        best = -1
        for off in np.ndindex(*([3] * d)):
            idx = [base[a] + off[a] - 1 for a in range(d)]
            if any(i < 0 or i >= nc[a] for a, i in enumerate(idx)):
                continue
            leaf = cells[tuple(idx)]
            b = bounds[leaf]
            if all(b[2 * a] <= x[a] <= b[2 * a + 1] for a in range(d)) and (best < 0 or leaf < best):
                best = leaf
        out[k] = max(best, 0)
    return out


@pytest.mark.parametrize("dim", [2, 3])
def test_cell_table_locates_the_first_containing_leaf(dim):
    if dim == 2:
        bounds = adaptive_bounds_2D()
    else:
        bounds = uniform_leaf_bounds_3D((0.0, 1.0, 0.0, 1.0, 0.0, 1.0), 2)
    cells, nc, lo, h = ip._cell_table(bounds, dim)
    rng = np.random.default_rng(dim)
    lo_b = bounds[:, 0::2].min(0)
    hi_b = bounds[:, 1::2].max(0)
    pts = rng.uniform(lo_b - 0.05, hi_b + 0.05, (300, dim))
    # points on leaf edges and corners, where several closed boxes meet
    edges = np.unique(np.concatenate([bounds[:, 2 * a:2 * a + 2].ravel() for a in range(dim)]))
    pts = np.concatenate([pts, rng.choice(edges, (200, dim))])
    assert np.array_equal(_locate_like_kernel(pts, bounds, cells, nc, lo, h),
                          O._first_containing_leaf(pts, bounds))


def test_leaf_node_weights_match_the_reference_formula():
    b = adaptive_bounds_2D()
    nodes, wts = ip._leaf_nodes(b, 7, 2)
    for leaf in range(len(b)):
        for a in range(2):
            assert np.allclose(wts[leaf, a], ip._bary_weights(nodes[leaf, a]), rtol=1e-15)
    c = O.chebyshev_points(7)
    assert np.allclose(nodes[0, 1], np.flip(O.affine_transform(c, b[0, 2:4])))

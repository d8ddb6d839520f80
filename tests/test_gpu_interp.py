"""GPU interpolation between the HPS grid and rectangular grids against the
oracle restatement of the reference (_interpolation_methods.py), and the
reference's own polynomial cases through Domain.interp_*."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300 import _interpolation as ip
from jaxhps_gb300._grid_creation_2D import bounds_to_cheby_points_2D, uniform_leaf_bounds_2D
from jaxhps_gb300._grid_creation_3D import bounds_to_cheby_points_3D, uniform_leaf_bounds_3D
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


def _adaptive_bounds_2D():
    top = uniform_leaf_bounds_2D((-1.0, 1.0, 3.0, 4.0), 1)
    sw = uniform_leaf_bounds_2D(tuple(top[0]), 1)
    return np.concatenate([sw, top[1:]])


def _rel(a, b):
    a = a.cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("kind,nsrc", [("uniform", None), ("uniform", 3), ("adaptive", None)])
def test_interp_from_hps_2D_matches_oracle(cuda, kind, nsrc):
    p = 8
    bounds = uniform_leaf_bounds_2D((-1.0, 1.0, 3.0, 4.0), 2) if kind == "uniform" else _adaptive_bounds_2D()
    pts = bounds_to_cheby_points_2D(bounds, p)
    rng = np.random.default_rng(5)
    f = np.sin(3 * pts[..., 0]) * np.cos(2 * pts[..., 1])
    if nsrc:
        f = np.stack([f * (k + 1) + rng.standard_normal(f.shape) * 0.1 for k in range(nsrc)], -1)
    # targets on leaf edges and corners
    xv = np.linspace(-1, 1, 9)
    yv = np.linspace(3.0, 4.0, 7)
    vals, tp = ip.interp_from_hps_2D(bounds, p, f, xv, yv)
    ref, tref = O.oracle_interp_from_hps(bounds, p, f, [xv, yv])
    assert vals.shape == ref.shape
    assert np.array_equal(tp, tref)
    assert _rel(vals, ref) < 1e-12
    # a target outside the box takes leaf 0, as in the reference; its value
    # is a far extrapolation whose normalising sum cancels, so rounding
    # differences grow to ~1e-3 there (another leaf would differ by O(1))
    out, _ = ip.interp_from_hps_2D(bounds, p, f, np.array([1.25]), np.array([3.1]))
    ref_out, _ = O.oracle_interp_from_hps(bounds, p, f, [np.array([1.25]), np.array([3.1])])
    assert _rel(out, ref_out) < 1e-2


def test_interp_from_hps_3D_matches_oracle(cuda):
    p = 5
    bounds = uniform_leaf_bounds_3D((0.0, 1.0, 0.0, 1.0, 0.0, 1.0), 1)
    pts = bounds_to_cheby_points_3D(bounds, p)
    f = np.exp(pts[..., 0]) * np.sin(2 * pts[..., 1] + pts[..., 2])
    ax = [np.linspace(0, 1, 5), np.linspace(0, 1, 4), np.linspace(0, 1, 3)]
    vals, tp = ip.interp_from_hps_3D(bounds, p, f, *ax)
    ref, tref = O.oracle_interp_from_hps(bounds, p, f, ax)
    assert vals.shape == ref.shape and np.array_equal(tp, tref)
    assert _rel(vals, ref) < 1e-12


@pytest.mark.parametrize("dim", [2, 3])
def test_interp_to_hps_matches_oracle(cuda, dim):
    # samples of a smooth function on Chebyshev-distributed nodes (random
    # nodes make the global interpolant's Lebesgue constant explode)
    if dim == 2:
        p, bounds = 7, _adaptive_bounds_2D()
        ax = [O.affine_transform(O.chebyshev_points(9), (-1, 1)), O.affine_transform(O.chebyshev_points(12), (3, 4))]
    else:
        p, bounds = 4, uniform_leaf_bounds_3D((0.0, 1.0, 0.0, 1.0, 0.0, 1.0), 1)
        ax = [O.affine_transform(O.chebyshev_points(n), (0, 1)) for n in (6, 7, 5)]
    G = np.meshgrid(*ax, indexing="ij")
    samples = np.cos(2 * G[0] + G[1]) * (1 + 0.5 * G[-1] ** 2)
    fn = ip.interp_to_hps_2D if dim == 2 else ip.interp_to_hps_3D
    out = fn(bounds, samples, p, *ax)
    ref = O.oracle_interp_to_hps(bounds, samples, p, ax)
    assert out.shape == ref.shape
    assert _rel(out, ref) < 1e-12


def test_domain_interp_from_interior_points_polynomial(cuda):
    """The reference's tests/test_domain.py Test_interp_from_interior_points."""
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=6, q=4, root=root, L=2)
    f = lambda x: x[..., 0] ** 2 - 3 * x[..., 1]   # noqa: E731
    xv = np.linspace(-1, 1, 3)
    samples, pts = dom.interp_from_interior_points(f(dom.interior_points), xv, xv)
    assert np.allclose(samples.numpy(), f(pts), atol=1e-12)


def test_domain_interp_to_interior_points_polynomial(cuda):
    """The reference's tests/test_domain.py Test_interp_to_interior_points
    (n_x != n_y catches exchanged axes), 2D and 3D."""
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=6, q=4, root=root, L=2)
    xv, yv = np.linspace(-1, 1, 10), np.linspace(-1, 1, 11)
    X, Y = np.meshgrid(xv, yv, indexing="ij")
    f = lambda x, y: x ** 2 - 3 * y   # noqa: E731
    out = dom.interp_to_interior_points(f(X, Y), xv, yv)
    exp = f(dom.interior_points[..., 0], dom.interior_points[..., 1])
    assert out.shape == exp.shape and np.allclose(out.numpy(), exp, atol=1e-11)
    root3 = hps.DiscretizationNode3D(-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    dom3 = hps.Domain(p=4, q=2, root=root3, L=1)
    ax = [np.linspace(-1, 1, 5), np.linspace(-1, 1, 6), np.linspace(-1, 1, 4)]
    G = np.stack(np.meshgrid(*ax, indexing="ij"), -1)
    g = lambda x: x[..., 0] * x[..., 1] - x[..., 2] ** 2   # noqa: E731
    out3 = dom3.interp_to_interior_points(g(G), *ax)
    assert np.allclose(out3.numpy(), g(dom3.interior_points), atol=1e-11)
    with pytest.raises(NotImplementedError):
        dom.interp_to_boundary_points(None, None, None)

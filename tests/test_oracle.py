"""Pins the FP64 oracle against the reference's own known-answer tests.

The reference stores no golden vectors; its accuracy tests
(tests/test_accuracy/*.py, tests/test_quadrature/test_differentiation.py)
pin results through analytic cases that the discretization reproduces to
rounding.  The same cases are re-run here against oracle/hps_oracle.py.
"""

import numpy as np
import pytest

from oracle import hps_oracle as O

PI = np.pi
ROOT = (-PI / 2, PI / 2, -PI / 2, PI / 2)   # tests/test_accuracy/cases.py:27-31
ATOL = 1e-12                                # test_local_solve_stage_accuracy.py:43


# --- analytic case "polynomial data with one non-zero source" (cases.py:47-139)
def g_poly(x):
    return x[..., 0] ** 2 - x[..., 1] ** 2


def src_poly(x):
    return 2 * x[..., 1] * (x[..., 1] ** 2 - (PI / 2) ** 2) + 6 * x[..., 1] * (x[..., 0] ** 2 - (PI / 2) ** 2)


def part_poly(x):
    return x[..., 1] * (x[..., 1] ** 2 - (PI / 2) ** 2) * (x[..., 0] ** 2 - (PI / 2) ** 2)


def dpart_dx(x):
    return 2 * x[..., 0] * x[..., 1] * (x[..., 1] ** 2 - (PI / 2) ** 2)


def dpart_dy(x):
    return (x[..., 0] ** 2 - (PI / 2) ** 2) * (3 * x[..., 1] ** 2 - (PI / 2) ** 2)


def outward_normal(bp, dfdx, dfdy):
    n = bp.shape[0] // 4
    return np.concatenate([-dfdy(bp[:n]), dfdx(bp[n:2 * n]), dfdy(bp[2 * n:3 * n]), -dfdx(bp[3 * n:])])


def test_differentiation_known_answers():
    """tests/test_quadrature/test_differentiation.py:11-81."""
    d2 = O.differentiation_matrix_1D(O.chebyshev_points(2))
    assert np.allclose(d2, [[-0.5, 0.5], [-0.5, 0.5]])
    d3 = O.differentiation_matrix_1D(O.chebyshev_points(3))
    assert np.allclose(d3, [[-1.5, 2, -0.5], [-0.5, 0, 0.5], [0.5, -2, 1.5]])
    d4 = O.differentiation_matrix_1D(O.chebyshev_points(4))
    exp4 = -np.array([[19 / 6, -4, 4 / 3, -0.5], [1, -1 / 3, -1, 1 / 3], [-1 / 3, 1, 1 / 3, -1],
                      [0.5, -4 / 3, 4, -19 / 6]])
    assert np.allclose(d4, exp4)
    x = O.chebyshev_points(7)
    assert np.allclose(O.differentiation_matrix_1D(x) @ x ** 2, 2 * x)


def test_interpolation_reproduces_polynomials():
    xs = O.gauss_points(9)
    ys = np.linspace(-1, 1, 13)
    m = O.barycentric_matrix_1D(xs, ys)
    assert np.allclose(m @ (xs ** 5 - 2 * xs), ys ** 5 - 2 * ys, atol=1e-13)
    # exact node hits give unit rows
    m2 = O.barycentric_matrix_1D(O.chebyshev_points(6), O.chebyshev_points(6))
    assert np.allclose(m2, np.eye(6))


def test_ext_first_order_small():
    """_grid_creation_2D.py:203-233 for n=3 gives [2,5,8,7,6,3,0,1,4]."""
    assert list(O.ext_first_order_2D(3)) == [2, 5, 8, 7, 6, 3, 0, 1, 4]


def test_leaf_dtn_known_answer():
    """check_leaf_accuracy_DtN (test_local_solve_stage_accuracy.py:134-260), p=16, q=14, L=0."""
    p, q = 16, 14
    pts = O.leaf_points_2D(O.uniform_leaf_bounds_2D(ROOT, 0), p)
    ones = np.ones(pts.shape[:2])
    pr = O.Problem2D(ROOT, 0, p, q, {"D_xx": ones, "D_yy": ones}, src_poly(pts))
    A = O.assemble_operator(pr.coeffs, pr.ops, 1, p * p)
    Y, T, v, h = O.leaf_dtn(A, pr.source, pr.P, pr.Q)
    bp = pr.boundary_points
    g = g_poly(bp)
    dn = outward_normal(bp, lambda x: 2 * x[..., 0], lambda x: -2 * x[..., 1])
    assert np.allclose(T[0] @ g, dn, atol=ATOL, rtol=0)
    assert np.allclose(Y[0] @ g, g_poly(pts[0]), atol=ATOL, rtol=0)
    assert np.allclose(v[0, :, 0], part_poly(pts[0]), atol=ATOL, rtol=0)
    assert np.allclose(h[0, :, 0], outward_normal(bp, dpart_dx, dpart_dy), atol=ATOL, rtol=0)


@pytest.mark.parametrize("L,p,q", [(1, 6, 4), (2, 8, 6), (3, 8, 6)])
def test_merge_dtn_known_answer(L, p, q):
    """check_merge_accuracy_2D_DtN_uniform (test_single_merge_accuracy.py:56-166),
    extended to several merge levels."""
    pts = O.leaf_points_2D(O.uniform_leaf_bounds_2D(ROOT, L), p)
    ones = np.ones(pts.shape[:2])
    pr = O.Problem2D(ROOT, L, p, q, {"D_xx": ones, "D_yy": ones}, src_poly(pts)).build()
    bp = pr.boundary_points
    dn = outward_normal(bp, lambda x: 2 * x[..., 0], lambda x: -2 * x[..., 1])
    assert np.allclose(pr.T_top @ g_poly(bp), dn, atol=1e-11, rtol=0)
    u = pr.solve(g_poly(bp))
    assert np.allclose(u, g_poly(pts) + part_poly(pts), atol=1e-12 * max(1, L), rtol=0)


# --- ItI analytic case with complex coefficients (cases.py:212-265)
CC = 1.0 + 0.1j


def u_cc(x):
    return x[..., 0] ** 3 + 3 * x[..., 1] ** 2


def f_cc(x):
    return 6 * x[..., 0] + 6 + CC * u_cc(x)


def imp_data(bp, eta, sign):
    dn = outward_normal(bp, lambda x: 3 * x[..., 0] ** 2, lambda x: 6 * x[..., 1])
    return dn + sign * 1j * eta * u_cc(bp)


def test_leaf_iti_known_answer():
    p, q, eta = 16, 14, 1.0
    pts = O.leaf_points_2D(O.uniform_leaf_bounds_2D(ROOT, 0), p)
    ones = np.ones(pts.shape[:2])
    pr = O.Problem2D(ROOT, 0, p, q, {"D_xx": ones, "D_yy": ones, "I": CC * ones}, f_cc(pts), iti=True, eta=eta)
    A = O.assemble_operator(pr.coeffs, pr.ops, 1, p * p)
    Y, T, v, h = O.leaf_iti(A, pr.source, pr.P, pr.QH, pr.G)
    bp = pr.boundary_points
    fin = imp_data(bp, eta, +1)
    assert np.allclose(T[0] @ fin + h[0, :, 0], imp_data(bp, eta, -1), atol=1e-10, rtol=0)
    assert np.allclose(Y[0] @ fin + v[0, :, 0], u_cc(pts[0]), atol=1e-10, rtol=0)


@pytest.mark.parametrize("L", [1, 2])
def test_merge_iti_known_answer(L):
    p, q, eta = 10, 8, 1.0
    pts = O.leaf_points_2D(O.uniform_leaf_bounds_2D(ROOT, L), p)
    ones = np.ones(pts.shape[:2])
    pr = O.Problem2D(ROOT, L, p, q, {"D_xx": ones, "D_yy": ones, "I": CC * ones}, f_cc(pts), iti=True,
                     eta=eta).build()
    bp = pr.boundary_points
    fin = imp_data(bp, eta, +1)
    assert np.allclose(pr.T_top @ fin + pr.h_top[:, 0], imp_data(bp, eta, -1), atol=1e-9, rtol=0)
    assert np.allclose(pr.solve(fin), u_cc(pts), atol=1e-10, rtol=0)


@pytest.mark.parametrize("L,p,q", [(1, 6, 4), (2, 6, 4)])
def test_oct_merge_known_answer(L, p, q):
    """3D analytic case: u = x^3 - 3 x y^2 + z^2 (Laplacian 2) is a degree-3
    polynomial, reproduced by the discretization for p >= 4, q >= 4 up to
    rounding through the leaf, oct-merge and down-pass restatements."""
    root = (-1.0, 1.0, -0.5, 1.5, 0.0, 2.0)
    pts = O.leaf_points_3D(O.uniform_leaf_bounds_3D(root, L), p)
    x, y, z = pts[..., 0], pts[..., 1], pts[..., 2]
    ones = np.ones_like(x)
    pr = O.Problem3D(root, L, p, q, {"D_xx": ones, "D_yy": ones, "D_zz": ones}, 2 * ones).build()
    bp = pr.boundary_points
    u = pr.solve(bp[:, 0] ** 3 - 3 * bp[:, 0] * bp[:, 1] ** 2 + bp[:, 2] ** 2)
    assert np.abs(u - (x ** 3 - 3 * x * y ** 2 + z ** 2)).max() < 1e-11


def test_oct_merge_known_answer_variable_coefficients():
    """(1 + x^2) u_xx + u_yy + u_zz + y u_z - u = f with u = x y + z^2 - y^3."""
    L, p, q = 1, 6, 4
    root = (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    pts = O.leaf_points_3D(O.uniform_leaf_bounds_3D(root, L), p)
    x, y, z = pts[..., 0], pts[..., 1], pts[..., 2]
    u = x * y + z ** 2 - y ** 3
    f = 0 + (-6 * y) + 2 + y * (2 * z) - u
    ones = np.ones_like(x)
    pr = O.Problem3D(root, L, p, q, {"D_xx": 1 + x ** 2, "D_yy": ones, "D_zz": ones, "D_z": y, "I": -ones}, f).build()
    bp = pr.boundary_points
    ub = pr.solve(bp[:, 0] * bp[:, 1] + bp[:, 2] ** 2 - bp[:, 1] ** 3)
    assert np.abs(ub - u).max() < 1e-11


def test_mlp_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n_par = 64 * 513 + 64 + 64 * 64 + 64 + 64 + 1
    params = rng.standard_normal(n_par) * 0.05
    X = rng.standard_normal((7, 513))
    y = (rng.random(7) > 0.5).astype(float)
    g = O.mlp_grad(params, X, y, pos_weight=2.5)
    for k in list(rng.choice(n_par, 40, replace=False)) + [n_par - 1, n_par - 2]:
        e = np.zeros(n_par)
        e[k] = 1e-6
        fd = (O.mlp_loss(params + e, X, y, 2.5) - O.mlp_loss(params - e, X, y, 2.5)) / 2e-6
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-8, k


def _adaptive_oracle_tree(q):
    root = O.OctNode((0, 1, 0, 1, 0, 1))
    O.oracle_add_eight_children(root, root, q)
    for ch in root.children:
        O.oracle_add_eight_children(ch, root, q)
    O.oracle_add_eight_children(root.children[0].children[1], root, q)
    O.oracle_add_eight_children(root.children[6].children[0], root, q)
    return root


def _oracle_root_boundary_points(root, q):
    fl = O.oracle_face_leaves(root)
    g = O.gauss_points(q)
    tang = ((1, 2), (1, 2), (0, 2), (0, 2), (0, 1), (0, 1))
    out = []
    for f in range(6):
        a, b = tang[f]
        for lf in fl[f]:
            U, V = np.meshgrid(O.affine_transform(g, lf.b[2 * a:2 * a + 2]), O.affine_transform(g, lf.b[2 * b:2 * b + 2]),
                               indexing="ij")
            P3 = np.empty((q * q, 3))
            P3[:, f // 2] = root.b[f]
            P3[:, a], P3[:, b] = U.ravel(), V.ravel()
            out.append(P3)
    return np.concatenate(out)


def test_adaptive_oracle_polynomial_known_answer():
    """A degree-3 solution is reproduced through compressed interfaces
    (L_1f4 / L_4f1 are exact on degree < q polynomials)."""
    p, q = 6, 4
    root = _adaptive_oracle_tree(q)
    leaves = root.leaves()
    pts = O.leaf_points_3D(np.array([lf.b for lf in leaves]), p)
    x, y, z = pts[..., 0], pts[..., 1], pts[..., 2]
    ones = np.ones_like(x)
    O.oracle_adaptive_build_3D(root, p, q, {"D_xx": ones, "D_yy": ones, "D_zz": ones, "D_x": y}, 2 * ones + y * (3 * x ** 2 - 3 * y ** 2))
    bp = _oracle_root_boundary_points(root, q)
    u = O.oracle_adaptive_solve_3D(root, bp[:, 0] ** 3 - 3 * bp[:, 0] * bp[:, 1] ** 2 + bp[:, 2] ** 2)
    assert np.abs(u[..., 0] - (x ** 3 - 3 * x * y ** 2 + z ** 2)).max() < 1e-11
    assert any(any(v) for v in root.flags.values())     # the tree exercises compression

"""CPU tests of the 3D host side: operators and grids against the oracle's
restatement of the reference's explicit formulas, the reference's operator
known answers (tests/test_precompute_operators_3D.py), and the oct-merge /
down-pass index maps against the oracle's block assembly."""

import numpy as np
import pytest

import jaxhps_gb300 as hps
from jaxhps_gb300 import _grid_creation_3D as g3
from jaxhps_gb300 import _index_maps as im
from jaxhps_gb300 import _precompute_operators_3D as op3
from jaxhps_gb300._quadrature import affine_transform, chebyshev_points, gauss_points
from oracle import hps_oracle as O
from test_host import _emulate_merge

PI2 = np.pi / 2


@pytest.mark.parametrize("p", [3, 4, 6, 10])
def test_face_indices_match_reference_formulas(p):
    for f in range(6):
        assert np.array_equal(op3.face_idxes(p, f), O.face_idxes_3D(p, f)), f
    assert np.array_equal(g3.rearrange_indices_ext_int(p), O.ext_first_order_3D(p))


@pytest.mark.parametrize("p,q", [(4, 2), (6, 4), (10, 8)])
def test_operators_3D_match_oracle(p, q):
    half = 0.41
    mine = op3.precompute_diff_operators_3D(p, half)
    ref = O.diff_operators_3D(p, half)
    for a, b in zip(mine, ref):
        assert np.allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(b).max())
    assert np.allclose(op3.precompute_P_3D_DtN(p, q), O.P_3D_DtN(p, q), atol=1e-14)
    assert np.allclose(op3.precompute_Q_3D_DtN(p, q, *mine[:3]), O.Q_3D_DtN(p, q, *ref[:3]), rtol=1e-12,
                       atol=1e-10)


def _cheby_pts(p, lo=-PI2, hi=PI2):
    return g3.bounds_to_cheby_points_3D(np.array([[lo, hi, lo, hi, lo, hi]]), p)[0]


def test_diff_operators_known_answers():
    """tests/test_precompute_operators_3D.py:42-165."""
    p = 5
    x = _cheby_pts(p)
    dx, dy, dz, dxx, dyy, dzz, dxy, dxz, dyz = op3.precompute_diff_operators_3D(p, PI2)
    f = x.sum(-1)
    for d in (dx, dy, dz):
        assert np.allclose(d @ f, 1.0)
    f = (x ** 2).sum(-1)
    for d, e in ((dxx, 2), (dyy, 2), (dzz, 2), (dxy, 0), (dxz, 0), (dyz, 0)):
        assert np.allclose(d @ f, e, atol=1e-10)
    f = x[:, 0] * x[:, 1] * x[:, 2]
    assert np.allclose(dxy @ f, x[:, 2]) and np.allclose(dxz @ f, x[:, 1]) and np.allclose(dyz @ f, x[:, 0])
    p = 16
    x = _cheby_pts(p)
    dx, dy, dz = op3.precompute_diff_operators_3D(p, PI2)[:3]
    f = np.sin(x).sum(-1)
    for k, d in enumerate((dx, dy, dz)):
        assert np.allclose(d @ f, np.cos(x[:, k]), atol=1e-8)


def test_P_Q_known_answers():
    """tests/test_precompute_operators_3D.py:177-373: interpolation of
    x + y + z from the boundary Gauss grid, normal derivatives of
    x^2 + 3y - xz."""
    p, q = 8, 6
    root = hps.DiscretizationNode3D(-PI2, PI2, -PI2, PI2, -PI2, PI2)
    x = _cheby_pts(p)
    gp = g3.compute_boundary_Gauss_points_uniform_3D(root, 0, q)
    P = op3.precompute_P_3D_DtN(p, q)
    n_cb = p ** 3 - (p - 2) ** 3
    assert np.allclose(P @ gp.sum(-1), x[:n_cb].sum(-1))
    dx, dy, dz = op3.precompute_diff_operators_3D(p, PI2)[:3]
    Q = op3.precompute_Q_3D_DtN(p, q, dx, dy, dz)
    f = x[:, 0] ** 2 + 3 * x[:, 1] - x[:, 0] * x[:, 2]
    dn = Q @ f
    n = q * q
    X, Z = gp[:, 0], gp[:, 2]
    exp = np.concatenate([-(2 * X[:n] - Z[:n]), 2 * X[n:2 * n] - Z[n:2 * n], -3 * np.ones(n), 3 * np.ones(n),
                          X[4 * n:5 * n], -X[5 * n:]])
    assert np.allclose(dn, exp)


def test_projection_ops_and_L8f1_reproduce_polynomials():
    q = 6
    g = gauss_points(q)
    L_4f1, L_1f4 = op3.precompute_projection_ops_3D(q)
    lo, hi = affine_transform(g, (-1, 0)), affine_transform(g, (0, 1))

    def f(u, v):
        return 1 + u - 2 * v + u * v + v ** 2

    U, V = np.meshgrid(g, g, indexing="ij")
    coarse = f(U.ravel(), V.ravel())
    fine = []
    for a, b in ((lo, lo), (hi, lo), (hi, hi), (lo, hi)):
        A, B = np.meshgrid(a, b, indexing="ij")
        fine.append(f(A.ravel(), B.ravel()))
    fine = np.concatenate(fine)
    assert np.allclose(L_4f1 @ coarse, fine)
    assert np.allclose(L_1f4 @ fine, coarse)
    with pytest.raises(ValueError):
        op3.precompute_projection_ops_3D(5)
    p = 5
    L8 = op3.precompute_L_8f1(p)
    parent = g3.bounds_to_cheby_points_3D(np.array([[-1, 1, -1, 1, -1, 1.0]]), p)[0]
    kids = g3.bounds_to_cheby_points_3D(g3.bounds_for_oct_subdivision((-1, 1, -1, 1, -1, 1.0)), p).reshape(-1, 3)

    def h(x):
        return x[:, 0] ** 2 * x[:, 1] - x[:, 2] ** 3 + x[:, 0] * x[:, 2]

    assert np.allclose(L8 @ h(parent), h(kids))


@pytest.mark.parametrize("L,p,q", [(0, 4, 2), (1, 5, 4), (2, 4, 2)])
def test_grids_3D_match_oracle(L, p, q):
    root = hps.DiscretizationNode3D(-1.0, 2.0, 0.0, 1.0, -0.5, 0.5)
    rb = root.bounds
    assert np.allclose(g3.compute_interior_Chebyshev_points_uniform_3D(root, L, p),
                       O.leaf_points_3D(O.uniform_leaf_bounds_3D(rb, L), p))
    assert np.allclose(g3.compute_boundary_Gauss_points_uniform_3D(root, L, q), O.boundary_gauss_points_3D(rb, L, q))


def _uniform_tree(root, L):
    if L == 0:
        return root
    kids = tuple(_uniform_tree(hps.DiscretizationNode3D(*b, depth=root.depth + 1), L - 1)
                 for b in g3.bounds_for_oct_subdivision(root.bounds))
    root.children = kids
    return root


def test_adaptive_grid_functions_on_a_uniform_tree():
    root = _uniform_tree(hps.DiscretizationNode3D(-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), 2)
    assert np.allclose(g3.compute_boundary_Gauss_points_adaptive_3D(root, 4),
                       g3.compute_boundary_Gauss_points_uniform_3D(root, 2, 4))
    assert np.allclose(g3.compute_interior_Chebyshev_points_adaptive_3D(root, 4),
                       g3.compute_interior_Chebyshev_points_uniform_3D(root, 2, 4))


def test_domain_3D_uniform():
    root = hps.DiscretizationNode3D(-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=6, q=4, root=root, L=2)
    assert dom.interior_points.shape == (64, 216, 3)
    assert dom.boundary_points.shape == (6 * 16 * 16, 3)


@pytest.mark.parametrize("nf", [1, 4])
def test_oct_merge_maps_reproduce_oracle(nf):
    rng = np.random.default_rng(nf)
    n = 6 * nf
    Ts = [rng.standard_normal((n, n)) + 6 * np.eye(n) for _ in range(8)]
    hs = [rng.standard_normal((n, 2)) for _ in range(8)]
    S, T, h, gt = O.oct_merge_dtn(Ts, hs)
    maps = im.oct_merge_maps_dtn(nf)
    S2, T2, h2, gt2 = _emulate_merge(Ts, hs, maps)
    assert np.allclose(S, S2) and np.allclose(T, T2) and np.allclose(h, h2) and np.allclose(gt, gt2)


@pytest.mark.parametrize("nf", [1, 4])
def test_oct_down_scatter_maps_reproduce_oracle(nf):
    rng = np.random.default_rng(3 + nf)
    S = rng.standard_normal((12 * nf, 24 * nf))
    g = rng.standard_normal((24 * nf, 2))
    gt = rng.standard_normal((12 * nf, 2))
    ref = O._propagate_down_oct(S, g, gt)
    maps = im.oct_merge_maps_dtn(nf)
    gi = S @ g + gt
    out = np.empty((8, 6 * nf, 2))
    for c in range(8):
        for k in range(6 * nf):
            cd = maps.code[c, k]
            out[c, k] = g[cd] if cd >= 0 else gi[-cd - 1]
    assert np.allclose(out, ref)


def test_leaf_gauss_nodes_3D_and_pairing():
    from jaxhps_gb300._refinement import node_maps

    root = hps.DiscretizationNode3D(-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    q = 4
    one = g3.leaf_boundary_gauss_points_3D(np.array([root.bounds]), q)[0]
    assert np.allclose(one, g3.compute_boundary_Gauss_points_uniform_3D(root, 0, q))
    dom = hps.Domain(p=6, q=q, root=root, L=2)
    nodes = g3.leaf_boundary_gauss_points_3D(g3.uniform_leaf_bounds_3D(root.bounds, 2), q)
    nbr, bnode = node_maps(nodes, dom.boundary_points, scale=2.0)
    flat = nodes.reshape(-1, 3)
    inner = nbr >= 0
    assert np.allclose(flat[inner], flat[nbr[inner]]) and (nbr[nbr[inner]] == np.nonzero(inner)[0]).all()
    assert (~inner).sum() == dom.boundary_points.shape[0]
    assert np.allclose(flat[bnode], dom.boundary_points)


def _oracle_leaf_boundary_data_3D(pr, bdry):
    S_lst = list(pr.S_lst[:-1]) + [pr.S_lst[-1][None]]
    g_lst = list(pr.g_lst[:-1]) + [pr.g_lst[-1][None]]
    g = bdry[None]
    for lvl in range(len(S_lst) - 1, -1, -1):
        g = np.concatenate([O._propagate_down_oct(S_lst[lvl][m], g[m], g_lst[lvl][m])
                            for m in range(S_lst[lvl].shape[0])])
    return g


def test_oracle_3D_solution_is_zero_of_dense_residual():
    """The discrete system the 3D mixed solver iterates on (collocation rows,
    flux continuity at paired Gauss nodes, Dirichlet data) is solved by the
    oracle's FP64 direct solution."""
    from jaxhps_gb300._refinement import node_maps

    L, p, q = 2, 6, 4
    rb = (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    rng = np.random.default_rng(4)
    pts = O.leaf_points_3D(O.uniform_leaf_bounds_3D(rb, L), p)
    c = 1 + 0.3 * np.exp(-(pts ** 2).sum(-1))
    ones = np.ones_like(c)
    f = rng.standard_normal(c.shape + (2,))
    pr = O.Problem3D(rb, L, p, q, {"D_xx": ones, "D_yy": ones, "D_zz": ones, "I": -c}, f).build()
    bdry = np.stack([np.sin(pr.boundary_points[:, 0]), pr.boundary_points[:, 2]], -1)
    u = pr.solve(bdry)
    gl = _oracle_leaf_boundary_data_3D(pr, bdry)
    A = O.assemble_operator(pr.coeffs, pr.ops, pts.shape[0], p ** 3)
    n_cb = pr.P.shape[0]
    u_full = np.concatenate([np.einsum("ab,lbs->las", pr.P, gl), u[:, n_cb:]], 1)
    r = f[:, n_cb:] - np.einsum("lab,lbs->las", A[:, n_cb:], u_full)
    assert np.abs(r).max() < 1e-9 * np.abs(f).max()
    flux = np.einsum("ab,lbs->las", pr.Q, u_full).reshape(-1, 2)
    nodes = g3.leaf_boundary_gauss_points_3D(g3.uniform_leaf_bounds_3D(rb, L), q)
    nbr, bnode = node_maps(nodes, pr.boundary_points, scale=2.0)
    inner = nbr >= 0
    assert np.abs(flux[inner] + flux[nbr[inner]]).max() < 1e-8 * np.abs(flux).max()
    assert np.allclose(gl.reshape(-1, 2)[bnode], bdry)

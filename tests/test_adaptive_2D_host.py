"""Adaptive 2D quadtrees, host side: tree editing and side point counts,
boundary leaf lists and Gauss points, interface compression lists, and the
oracle pinned by a quadratic known-answer case on a 2:1 tree."""

import numpy as np

from oracle import hps_oracle as O
from jaxhps_gb300._discretization_tree import DiscretizationNode2D, get_all_leaves
from jaxhps_gb300._discretization_tree_operations_2D import add_four_children, get_ordered_lst_of_boundary_nodes
from jaxhps_gb300._grid_creation_2D import compute_boundary_Gauss_points_adaptive_2D
from jaxhps_gb300 import _adaptive as ad


def product_tree(q):
    root = DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    add_four_children(root, root=root, q=q)
    a, b, c, d = root.children
    add_four_children(a, root=root, q=q)
    add_four_children(a.children[0], root=root, q=q)
    add_four_children(c, root=root, q=q)
    return root


def oracle_tree():
    root = O.QuadNode((-1.0, 1.0, -1.0, 1.0))
    a, b, c, d = root.split()
    a.split()
    a.children[0].split()
    c.split()
    return root


def oracle_bdry_points(root, q):
    s, e, n, w = O.oracle_side_leaves_2D(root)
    gq = O.gauss_points(q)
    x0, x1, y0, y1 = root.b
    return np.concatenate([np.stack([O.affine_transform(gq, lf.b[0:2]), np.full(q, y0)], -1) for lf in s] +
                          [np.stack([np.full(q, x1), O.affine_transform(gq, lf.b[2:4])], -1) for lf in e] +
                          [np.stack([O.affine_transform(gq, (lf.b[1], lf.b[0])), np.full(q, y1)], -1) for lf in n] +
                          [np.stack([np.full(q, x0), O.affine_transform(gq, (lf.b[3], lf.b[2]))], -1) for lf in w])


def test_side_counts_and_boundary_lists_match_the_leaves():
    q = 4
    root, oroot = product_tree(q), oracle_tree()
    for node, onode in [(root, oroot)] + list(zip(root.children, oroot.children)):
        lists = get_ordered_lst_of_boundary_nodes(node)
        olists = O.oracle_side_leaves_2D(onode)
        for s in range(4):
            assert [lf.bounds for lf in lists[s]] == [lf.b for lf in olists[s]]
        assert [node.n_0, node.n_1, node.n_2, node.n_3] == [q * len(x) for x in olists]
    assert np.allclose(compute_boundary_Gauss_points_adaptive_2D(root, q), oracle_bdry_points(oroot, q))


def test_interface_compression_lists_match_the_oracle():
    q = 4
    root, oroot = product_tree(q), oracle_tree()
    proj = ad.projection_lists(root)
    sl = [O.oracle_side_leaves_2D(k) for k in oroot.children]
    a5, b5 = O._compress_list_2D(sl[0][1], sl[1][3][::-1])
    d8, a8 = O._compress_list_2D(sl[3][0], sl[0][2][::-1])
    # the product keeps each side's flags in the side's own order
    assert list(proj[(0, 1)]) == a5 and list(proj[(1, 3)]) == b5[::-1]
    assert list(proj[(3, 0)]) == d8 and list(proj[(0, 2)]) == a8[::-1]
    assert any(a5) or any(b5)


def test_oracle_adaptive_2D_quadratic_known_answer():
    p, q = 8, 6
    root = oracle_tree()
    pts = O.leaf_points_2D(np.array([lf.b for lf in root.leaves()]), p)
    u = lambda x: x[..., 0] ** 2 - 2 * x[..., 1] ** 2 + x[..., 0] * x[..., 1] + 3   # noqa: E731
    cc = 1.0 + 0.5 * np.sin(pts[..., 0])
    f = 2 - 4 + cc * u(pts)
    O.oracle_adaptive_build_2D(root, p, q, {"D_xx": np.ones_like(cc), "D_yy": np.ones_like(cc), "I": cc}, f)
    sol = O.oracle_adaptive_solve_2D(root, u(oracle_bdry_points(root, q)), q)
    assert np.abs(sol[..., 0] - u(pts)).max() < 1e-10

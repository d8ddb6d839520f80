"""CPU tests of adaptive octree meshing: the oracle restatement against the
reference's own meshing tests (tests/test_adaptive_discretization_3D.py),
and the host tree operations against the reference's tree tests
(tests/test_discretization_tree_operations_3D.py)."""

import numpy as np
import pytest

import jaxhps_gb300 as hps
from jaxhps_gb300 import _adaptive_discretization_3D as ad
from jaxhps_gb300 import _discretization_tree_operations_3D as to
from jaxhps_gb300._discretization_tree import get_all_leaves
from oracle import hps_oracle as O


def _poly(x):
    return x[..., 1] + x[..., 0] ** 2


@pytest.mark.parametrize("p,l2", [(4, False), (6, True)])
def test_oracle_mesh_keeps_polynomial(p, l2):
    """tests/test_adaptive_discretization_3D.py:17-64: y + x^2 needs no refinement."""
    root = O.OctNode((0, 1, 0, 1, 0, 1))
    O.oracle_add_eight_children(root)
    O.oracle_adaptive_mesh_3D(root, _poly, 1e-3, p, p - 2, l2=l2)
    leaves = root.leaves()
    assert len(leaves) == 8 and all(lf.depth == 1 for lf in leaves)


def test_oracle_mesh_refines_a_bump_with_balance():
    def f(x):
        return np.exp(-((x - 0.3) ** 2).sum(-1) / 0.01)
    root = O.OctNode((0, 1, 0, 1, 0, 1))
    O.oracle_adaptive_mesh_3D(root, f, 1e-3, 6, 4)
    leaves = root.leaves()
    assert len(leaves) > 8
    # 2:1 balance across faces
    for a in leaves:
        for b in leaves:
            sa, sb = a.b[1] - a.b[0], b.b[1] - b.b[0]
            touch = all(min(a.b[2 * k + 1], b.b[2 * k + 1]) >= max(a.b[2 * k], b.b[2 * k]) for k in range(3))
            overlap = sum(min(a.b[2 * k + 1], b.b[2 * k + 1]) > max(a.b[2 * k], b.b[2 * k]) for k in range(3))
            if touch and overlap == 2:
                assert max(sa, sb) / min(sa, sb) <= 2 + 1e-12


def test_face_counts_uniform_and_nonuniform():
    """tests/test_discretization_tree_operations_3D.py:87-143."""
    q = 4
    root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
    to.add_eight_children(root, root=root, q=q)
    for ch in root.children:
        to.add_eight_children(ch, root=root, q=q)
        for gch in ch.children:
            to.add_eight_children(gch, root=root, q=q)
    assert [root.n_0, root.n_1, root.n_2, root.n_3, root.n_4, root.n_5] == [64 * q * q] * 6
    root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
    to.add_eight_children(root, root=root, q=q)
    to.add_eight_children(root.children[0], root=root, q=q)
    to.add_eight_children(root.children[0].children[0], root=root, q=q)
    assert (root.n_1, root.n_3, root.n_4) == (4 * q * q,) * 3
    assert (root.n_0, root.n_2, root.n_5) == (10 * q * q,) * 3
    oroot = O.OctNode((0, 1, 0, 1, 0, 1))
    O.oracle_add_eight_children(oroot, oroot, q)
    O.oracle_add_eight_children(oroot.children[0], oroot, q)
    O.oracle_add_eight_children(oroot.children[0].children[0], oroot, q)
    assert oroot.n == [root.n_0, root.n_1, root.n_2, root.n_3, root.n_4, root.n_5]


def test_find_path_and_interfaces():
    root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
    to.add_eight_children(root, root=root, q=3)
    to.add_eight_children(root.children[0], root=root, q=3)
    assert len(to.find_path_from_root_3D(root, root.children[0].children[0])) == 2
    root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
    for _ in range(3):
        for leaf in get_all_leaves(root):
            to.add_eight_children(leaf, root=root, q=4)
    for kw in ({"xval": 0.5}, {"yval": 0.25}):
        neg, pos = to.find_nodes_along_interface_3D(root, **kw)
        assert len(neg) == len(pos) == 4 ** 3
    neg, pos = to.find_nodes_along_interface_3D(root, yval=0.25)
    assert all(n.ymax == 0.25 for n in neg) and all(n.ymin == 0.25 for n in pos)
    with pytest.raises(ValueError):
        to.find_nodes_along_interface_3D(root, xval=0.5, yval=0.5)


def test_find_or_add_child_enforces_balance():
    root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
    to.add_eight_children(root, root=root, q=2)
    a = root.children[0]
    to.add_eight_children(a, root=root, q=2)
    ab = a.children[1]   # a's child b touches the x = 0.5 face
    to.add_eight_children(ab, root=root, q=2)
    vols = ad.volumes_to_check(ab, root)
    added = [ad.find_or_add_child(root, root, 2, *v) for v in vols]
    # the neighbour of a.b across x = 0.5 is root child b, which gets refined
    assert any(n is root.children[1] for n in added if n is not None)
    assert len(root.children[1].children) == 8


def test_dense_linf_check_helper_matches_oracle_operator():
    p = 5
    rng = np.random.default_rng(0)
    f0 = rng.standard_normal(p ** 3)
    L8 = O.L_8f1(p)
    f1 = L8 @ f0 + 1e-7
    ok, nrm = ad.check_current_discretization_global_linf_norm(f0, f1, L8, 1e-5, 0.1)
    assert ok and nrm == max(0.1, np.abs(f1).max())
    from jaxhps_gb300._precompute_operators_3D import precompute_L_8f1
    assert np.allclose(precompute_L_8f1(p), L8, atol=1e-13)

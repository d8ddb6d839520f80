"""GPU tests of adaptive octree meshing: the batched point generation and
tensor-product interpolation check against the oracle's dense L_8f1 check,
and whole meshes against the oracle restatement of the reference's meshing
(same leaves, same face point counts)."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300 import _adaptive_discretization_3D as ad
from jaxhps_gb300._discretization_tree import get_all_leaves
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


def _xp(x):
    return torch if isinstance(x, torch.Tensor) else np


def bump(x):
    xp = _xp(x)
    return xp.exp(-((x[..., 0] - 0.3) ** 2 + (x[..., 1] - 0.35) ** 2 + (x[..., 2] - 0.4) ** 2) / 0.01)


def front(x):
    xp = _xp(x)
    r = xp.sqrt(((x + 0.05) ** 2).sum(-1))
    return xp.arctan(20 * (r - 0.7))


def test_points_and_check_match_dense_oracle(cuda):
    p = 6
    rng = np.random.default_rng(0)
    lo = rng.uniform(-1, 0.5, (5, 3))
    side = rng.uniform(0.1, 0.5, (5, 1))
    bounds = np.stack([lo[:, 0], lo[:, 0] + side[:, 0], lo[:, 1], lo[:, 1] + side[:, 0], lo[:, 2],
                       lo[:, 2] + side[:, 0]], -1)
    consts = ad._CheckConstants(p, cuda)
    pts = ad.refinement_points(bounds, consts, cuda).cpu().numpy()
    for i, b in enumerate(bounds):
        assert np.allclose(pts[i, 0], O.leaf_points_3D(np.array([b]), p)[0], rtol=0, atol=1e-15)
        assert np.allclose(pts[i, 1:].reshape(-1, 3), O.leaf_points_3D(O.oct_children_bounds(b), p).reshape(-1, 3),
                           rtol=0, atol=1e-15)
    diff, ref, l2 = ad.refinement_check(bounds, front, consts, cuda, want_l2=True)
    L8 = O.L_8f1(p)
    r = O.ext_first_order_3D(p)
    for i, b in enumerate(bounds):
        f0 = front(O.leaf_points_3D(np.array([b]), p)[0])
        kids = O.oct_children_bounds(b)
        f1 = front(O.leaf_points_3D(kids, p).reshape(-1, 3))
        d = L8 @ f0 - f1
        assert np.isclose(diff[i], np.abs(d).max(), rtol=1e-12, atol=1e-15)
        assert np.isclose(ref[i], np.abs(f1).max(), rtol=1e-14)
        l2r = 0.0
        for k in range(8):
            w = np.einsum("i,j,k->ijk", O.chebyshev_weights(p, kids[k][0:2]), O.chebyshev_weights(p, kids[k][2:4]),
                          O.chebyshev_weights(p, kids[k][4:6])).ravel()[r]
            l2r += np.sum(w * d[k * p ** 3:(k + 1) * p ** 3] ** 2)
        assert np.isclose(l2[i], l2r, rtol=1e-10)


def _leaf_set(leaves, key):
    return sorted(tuple(round(v, 12) for v in key(lf)) for lf in leaves)


@pytest.mark.parametrize("fn,tol,l2,pre", [(bump, 1e-3, False, False), (bump, 1e-4, True, True),
                                           (front, 1e-3, False, True)])
def test_mesh_matches_oracle(cuda, fn, tol, l2, pre):
    p, q = 6, 4
    root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
    oroot = O.OctNode((0, 1, 0, 1, 0, 1))
    if pre:
        from jaxhps_gb300._discretization_tree_operations_3D import add_eight_children
        add_eight_children(root, root=root, q=q)
        O.oracle_add_eight_children(oroot, oroot, q)
    stats = {}
    ad.generate_adaptive_mesh_level_restriction(root, fn, tol, p, q, l2_norm=l2, stats=stats)
    O.oracle_adaptive_mesh_3D(oroot, fn, tol, p, q, l2=l2)
    mine = get_all_leaves(root)
    ref = oroot.leaves()
    assert len(mine) == len(ref) > 8
    assert [lf.bounds for lf in mine] == [r.b for r in ref]     # same leaves in the same order
    assert [lf.depth for lf in mine] == [r.depth for r in ref]
    assert [root.n_0, root.n_1, root.n_2, root.n_3, root.n_4, root.n_5] == oroot.n
    assert stats["leaves"] == len(mine) and stats["checked"] >= len(mine)


def test_domain_from_adaptive_discretization_3D(cuda):
    root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
    dom = hps.Domain.from_adaptive_discretization(p=6, q=4, root=root, f=bump, tol=1e-3)
    n = len(get_all_leaves(root))
    assert dom.interior_points.shape == (n, 216, 3)
    assert dom.boundary_points.shape[0] == root.n_0 + root.n_1 + root.n_2 + root.n_3 + root.n_4 + root.n_5
    lst = dom.get_adaptive_boundary_data_lst(lambda x: x[..., 0])
    assert [len(a) for a in lst] == [root.n_0, root.n_1, root.n_2, root.n_3, root.n_4, root.n_5]

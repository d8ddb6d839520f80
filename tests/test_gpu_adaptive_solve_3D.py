"""GPU parity of the adaptive 3D DtN build/solve (leaf stage with per-leaf
scaling, merges with interface compression, down pass with expansion)
against the oracle's restatement of the reference, plus an analytic case
and the uniform path as a reference on a uniformly refined tree.
Tolerance: relative max error <= 1e-11."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300._discretization_tree import get_all_leaves
from jaxhps_gb300._discretization_tree_operations_3D import add_eight_children
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _trees(q, extra=()):
    """Uniform depth-2 octree plus refinements of the given depth-2 nodes
    (all leaves at depth 2 or 3: 2:1 balanced)."""
    root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
    oroot = O.OctNode((0, 1, 0, 1, 0, 1))
    add_eight_children(root, root=root, q=q)
    O.oracle_add_eight_children(oroot, oroot, q)
    for i in range(8):
        add_eight_children(root.children[i], root=root, q=q)
        O.oracle_add_eight_children(oroot.children[i], oroot, q)
    for path in extra:
        n, o = root, oroot
        for k in path:
            n, o = n.children[k], o.children[k]
        add_eight_children(n, root=root, q=q)
        O.oracle_add_eight_children(o, oroot, q)
    return root, oroot


@pytest.mark.parametrize("extra,nsrc", [(((0, 1), (6, 0)), None), (((0, 1), (0, 2), (3, 5), (5, 1), (7, 3)), 2)])
def test_adaptive_build_solve_matches_oracle(cuda, extra, nsrc):
    p, q = 6, 4
    root, oroot = _trees(q, extra)
    dom = hps.Domain(p=p, q=q, root=root)
    x = dom.interior_points
    rng = np.random.default_rng(len(extra))
    c = 1.0 + 0.3 * np.exp(-((x - 0.4) ** 2).sum(-1) / 0.05)
    ones = np.ones_like(c)
    f = rng.standard_normal(x.shape[:2] + ((nsrc,) if nsrc else ()))
    kw = dict(D_xx_coefficients=ones, D_yy_coefficients=ones, D_zz_coefficients=ones, I_coefficients=c,
              D_y_coefficients=0.3 * x[..., 2])
    pde = hps.PDEProblem(dom, source=f, **kw)
    T_top = hps.build_solver(pde, return_top_T=True)
    bl = dom.get_adaptive_boundary_data_lst(lambda pts: np.sin(pts[..., 0]) + pts[..., 1] * pts[..., 2])
    if nsrc:
        bl = [np.stack([b * (k + 1) for k in range(nsrc)], -1) for b in bl]
    u = hps.solve(pde, bl)
    O.oracle_adaptive_build_3D(oroot, p, q, {"D_xx": ones, "D_yy": ones, "D_zz": ones, "I": c, "D_y": 0.3 * x[..., 2]},
                               f)
    ur = O.oracle_adaptive_solve_3D(oroot, np.concatenate(bl))
    if not nsrc:
        ur = ur[..., 0]
    assert tuple(u.shape) == ur.shape
    assert _rel(u, ur) < 1e-11
    assert _rel(T_top, oroot.T) < 1e-10
    assert T_top.shape[0] == sum([root.n_0, root.n_1, root.n_2, root.n_3, root.n_4, root.n_5])


def test_adaptive_path_on_uniform_tree_equals_uniform_path(cuda):
    p, q = 6, 4
    root, _ = _trees(q)
    dom_a = hps.Domain(p=p, q=q, root=root)
    dom_u = hps.Domain(p=p, q=q, root=hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0), L=2)
    x = dom_u.interior_points
    assert np.allclose(dom_a.interior_points, x)
    assert np.allclose(dom_a.boundary_points, dom_u.boundary_points)
    ones = np.ones(x.shape[:2])
    f = np.cos(3 * x[..., 0]) * x[..., 1]
    kw = dict(D_xx_coefficients=ones, D_yy_coefficients=ones, D_zz_coefficients=ones, I_coefficients=-2 * ones)
    pa, pu = hps.PDEProblem(dom_a, source=f, **kw), hps.PDEProblem(dom_u, source=f, **kw)
    hps.build_solver(pa)
    hps.build_solver(pu)
    g = np.exp(dom_u.boundary_points[:, 2])
    ua = hps.solve(pa, dom_a.get_adaptive_boundary_data_lst(lambda pts: np.exp(pts[..., 2])))
    uu = hps.solve(pu, g)
    assert _rel(ua, uu.numpy()) < 1e-11


def test_adaptive_polynomial_known_answer_gpu(cuda):
    p, q = 6, 4
    root, _ = _trees(q, ((0, 1), (6, 0)))
    dom = hps.Domain(p=p, q=q, root=root)
    x = dom.interior_points
    ones = np.ones(x.shape[:2])
    pde = hps.PDEProblem(dom, source=2 * ones, D_xx_coefficients=ones, D_yy_coefficients=ones, D_zz_coefficients=ones)
    hps.build_solver(pde)
    u = hps.solve(pde, dom.get_adaptive_boundary_data_lst(
        lambda pts: pts[..., 0] ** 3 - 3 * pts[..., 0] * pts[..., 1] ** 2 + pts[..., 2] ** 2)).numpy()
    assert np.abs(u - (x[..., 0] ** 3 - 3 * x[..., 0] * x[..., 1] ** 2 + x[..., 2] ** 2)).max() < 1e-10


def test_mesh_then_solve_wavefront(cuda):
    """Meshing, build and solve on a sharp front; the solution matches the
    manufactured one to the meshing tolerance's order."""
    p, q = 8, 6
    k, R, c0 = 10.0, 0.6, np.array([-0.05, -0.05, -0.05])

    def u_fn(x):
        xp = torch if isinstance(x, torch.Tensor) else np
        r = xp.sqrt(((x[..., 0] - c0[0]) ** 2 + (x[..., 1] - c0[1]) ** 2 + (x[..., 2] - c0[2]) ** 2))
        return xp.arctan(k * (r - R))

    def f_fn(x):
        xp = torch if isinstance(x, torch.Tensor) else np
        r = xp.sqrt(((x[..., 0] - c0[0]) ** 2 + (x[..., 1] - c0[1]) ** 2 + (x[..., 2] - c0[2]) ** 2))
        s = k * (r - R)
        return -2 * k * k * s / (1 + s * s) ** 2 + 2 * k / ((1 + s * s) * r)

    root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
    dom = hps.Domain.from_adaptive_discretization(p=p, q=q, root=root, f=f_fn, tol=1e-3)
    depths = {lf.depth for lf in get_all_leaves(root)}
    assert len(depths) > 1                       # a genuinely non-uniform tree
    x = dom.interior_points
    ones = np.ones(x.shape[:2])
    pde = hps.PDEProblem(dom, source=f_fn(x), D_xx_coefficients=ones, D_yy_coefficients=ones, D_zz_coefficients=ones)
    hps.build_solver(pde)
    u = hps.solve(pde, dom.get_adaptive_boundary_data_lst(u_fn)).numpy()
    assert np.abs(u - u_fn(x)).max() < 1e-3

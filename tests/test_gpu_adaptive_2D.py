"""Adaptive 2D quadtrees on the GPU: build + solve against the oracle
restatement of the reference's adaptive merges and down pass, the
quadratic known answer through the public API, and the GPU meshing against
the oracle's meshing (identical trees)."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300._discretization_tree_operations_2D import add_four_children
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


def product_tree(q, refine_c=True):
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    add_four_children(root, root=root, q=q)
    a, b, c, d = root.children
    add_four_children(a, root=root, q=q)
    add_four_children(a.children[0], root=root, q=q)
    if refine_c:
        add_four_children(c, root=root, q=q)
        add_four_children(c.children[2], root=root, q=q)
    return root


def oracle_tree(refine_c=True):
    root = O.QuadNode((-1.0, 1.0, -1.0, 1.0))
    a, b, c, d = root.split()
    a.split()
    a.children[0].split()
    if refine_c:
        c.split()
        c.children[2].split()
    return root


@pytest.mark.parametrize("nsrc", [None, 3])
def test_adaptive_2D_solve_matches_oracle(cuda, nsrc):
    p, q = 10, 8
    root = product_tree(q)
    dom = hps.Domain(p=p, q=q, root=root)
    x = dom.interior_points
    c = 1.0 + 0.5 * np.exp(-((x - 0.3) ** 2).sum(-1))
    rng = np.random.default_rng(7)
    shape = x.shape[:2] + ((nsrc,) if nsrc else ())
    f = np.sin(2 * x[..., 0])[..., None] * rng.uniform(0.5, 1.5, shape[2:] or (1,)) if nsrc else np.sin(2 * x[..., 0])
    ones = np.ones_like(c)
    pde = hps.PDEProblem(dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c)
    hps.build_solver(pde)
    bp = dom.boundary_points
    g = np.cos(bp[:, 0]) + bp[:, 1] ** 2
    if nsrc:
        g = np.stack([g * (k + 1) for k in range(nsrc)], -1)
    r = dom.root
    masks = [bp[:, 1] == r.ymin, bp[:, 0] == r.xmax, bp[:, 1] == r.ymax, bp[:, 0] == r.xmin]
    u = hps.solve(pde, [g[m] for m in masks])
    oroot = oracle_tree()
    O.oracle_adaptive_build_2D(oroot, p, q, {"D_xx": ones, "D_yy": ones, "I": c}, f)
    ur = O.oracle_adaptive_solve_2D(oroot, g, q)
    ur = ur if nsrc else ur[..., 0]
    u = u.numpy()
    assert u.shape == ur.shape
    assert np.abs(u - ur).max() / np.abs(ur).max() < 1e-10


def test_adaptive_2D_quadratic_known_answer(cuda):
    p, q = 8, 6
    root = product_tree(q)
    dom = hps.Domain(p=p, q=q, root=root)
    x = dom.interior_points
    uf = lambda y: y[..., 0] ** 2 - 2 * y[..., 1] ** 2 + y[..., 0] * y[..., 1] + 3   # noqa: E731
    c = 1.0 + 0.5 * np.sin(x[..., 0])
    ones = np.ones_like(c)
    pde = hps.PDEProblem(dom, source=-2 + c * uf(x), D_xx_coefficients=ones, D_yy_coefficients=ones,
                         I_coefficients=c)
    hps.build_solver(pde)
    u = hps.solve(pde, dom.get_adaptive_boundary_data_lst(uf))
    assert np.abs(u.numpy() - uf(x)).max() < 1e-10


@pytest.mark.parametrize("l2", [False, True])
def test_adaptive_2D_meshing_matches_oracle(cuda, l2):
    p, q, tol = 10, 8, 1e-4 if not l2 else 1e-5

    def front(y):
        if isinstance(y, torch.Tensor):
            return torch.atan(20 * (torch.sqrt(((y + 0.05) ** 2).sum(-1)) - 0.7))
        return np.arctan(20 * (np.sqrt(((y + 0.05) ** 2).sum(-1)) - 0.7))

    root = hps.DiscretizationNode2D(0.0, 1.0, 0.0, 1.0)
    dom = hps.Domain.from_adaptive_discretization(p=p, q=q, root=root, f=front, tol=tol, use_l_2_norm=l2)
    oroot = O.QuadNode((0.0, 1.0, 0.0, 1.0))
    O.oracle_adaptive_mesh_2D(oroot, front, tol, p, l2=l2)
    got = [lf.bounds for lf in hps.get_all_leaves(dom.root)]
    exp = [lf.b for lf in oroot.leaves()]
    assert got == exp
    assert len(got) > 10
    # the meshed domain solves: a quadratic through the public API
    x = dom.interior_points
    uf = lambda y: y[..., 0] * y[..., 1] + y[..., 0] ** 2   # noqa: E731
    ones = np.ones(x.shape[:2])
    pde = hps.PDEProblem(dom, source=2 * ones, D_xx_coefficients=ones, D_yy_coefficients=ones)
    hps.build_solver(pde)
    u = hps.solve(pde, dom.get_adaptive_boundary_data_lst(uf))
    assert np.abs(u.numpy() - uf(x)).max() < 1e-9

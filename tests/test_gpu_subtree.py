"""The subtree-recomputation API (solve_subtree, upward_pass_subtree,
downward_pass_subtree) gives the build_solver + solve results, DtN and ItI."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("iti", [False, True])
def test_subtree_api_matches_build_and_solve(cuda, iti):
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=8, q=6, root=root, L=3)
    x = dom.interior_points
    ones = np.ones(x.shape[:2])
    rng = np.random.default_rng(1)
    f = rng.standard_normal(x.shape[:2])
    kw = dict(source=f, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=(9.0 if iti else 1.0) * ones)
    if iti:
        kw.update(use_ItI=True, eta=3.0)
        f = f + 0j
    g = np.sin(dom.boundary_points[:, 0]) + (1j * dom.boundary_points[:, 1] if iti else 0)
    ref_pde = hps.PDEProblem(dom, **kw)
    T_ref = hps.build_solver(ref_pde, return_top_T=True)
    u_ref = hps.solve(ref_pde, g).numpy()
    u1 = hps.solve_subtree(hps.PDEProblem(dom, **kw), g).numpy()
    assert np.abs(u1 - u_ref).max() <= 1e-12 * np.abs(u_ref).max()
    pde = hps.PDEProblem(dom, **kw)
    T = hps.upward_pass_subtree(pde).numpy()
    assert np.abs(T - T_ref.cpu().numpy()).max() <= 1e-12 * np.abs(T).max()
    n = dom.boundary_points.shape[0] // 4
    u2 = hps.downward_pass_subtree(pde, [torch.as_tensor(g[k * n:(k + 1) * n]) for k in range(4)]).numpy()
    assert np.abs(u2 - u_ref).max() <= 1e-12 * np.abs(u_ref).max()

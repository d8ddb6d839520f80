"""Build once without a source, solve for many sources: the up pass with the
stored D^-1 and B D^-1 against the FP64 oracle given the source at build
time (the reference's source vs no-source agreement,
tests/test_accuracy/test_nosource_accuracy.py), DtN and ItI.
Tolerance: relative max error <= 1e-11."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300 import _nosource as ns_
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _dom(L, p, q):
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    return root, hps.Domain(p=p, q=q, root=root, L=L)


@pytest.mark.parametrize("L,p,q,nsrc", [(2, 8, 6, None), (3, 10, 8, 3)])
def test_nosource_dtn_matches_oracle(cuda, L, p, q, nsrc):
    root, dom = _dom(L, p, q)
    x = dom.interior_points
    c = 1.0 + 0.5 * np.exp(-((x[..., 0] - 0.2) ** 2 + (x[..., 1] + 0.3) ** 2) / 0.04)
    ones = np.ones_like(c)
    pde = hps.PDEProblem(dom, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c)
    T_top = hps.build_solver(pde, return_top_T=True)
    assert pde.Phi is not None and len(pde.D_inv_lst) == len(pde.BD_inv_lst) == L
    rng = np.random.default_rng(L)
    g = np.cos(dom.boundary_points[:, 0]) + dom.boundary_points[:, 1]
    for trial in range(2):          # several sources on one build
        f = rng.standard_normal(x.shape[:2] + ((nsrc,) if nsrc else ()))
        gg = np.stack([g * (k + 1) for k in range(nsrc)], -1) if nsrc else g
        u = hps.solve(pde, gg, source=f)
        ref = O.Problem2D(root.bounds, L, p, q, {"D_xx": ones, "D_yy": ones, "I": c}, f).build()
        assert _rel(u, ref.solve(gg)) < 1e-11
    assert _rel(T_top, ref.T_top) < 1e-10


def test_nosource_iti_matches_oracle(cuda):
    L, p, q, eta = 2, 10, 8, 4.0
    root, dom = _dom(L, p, q)
    x = dom.interior_points
    Icoef = 36.0 * (1 + 0.5 * np.exp(-((x[..., 0] - 0.2) ** 2 + (x[..., 1] + 0.3) ** 2) / 0.05))
    ones = np.ones_like(Icoef)
    pde = hps.PDEProblem(dom, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=Icoef, use_ItI=True,
                         eta=eta)
    hps.build_solver(pde)
    rng = np.random.default_rng(9)
    f = rng.standard_normal(x.shape[:2]) + 1j * rng.standard_normal(x.shape[:2])
    g = np.exp(1j * dom.boundary_points[:, 0])
    u = hps.solve(pde, g, source=f)
    ref = O.Problem2D(root.bounds, L, p, q, {"D_xx": ones, "D_yy": ones, "I": Icoef}, f, iti=True, eta=eta).build()
    assert _rel(u, ref.solve(g)) < 1e-11
    # h_last: the outgoing data of the particular solution on the root boundary
    v, g_lst, h_last = ns_.up_pass_uniform_2D_ItI(f, pde, return_h_last=True)
    assert _rel(h_last, ref.h_top[..., 0]) < 1e-10


def test_source_at_solve_needs_a_nosource_build(cuda):
    root, dom = _dom(1, 6, 4)
    x = dom.interior_points
    ones = np.ones(x.shape[:2])
    pde = hps.PDEProblem(dom, source=ones, D_xx_coefficients=ones, D_yy_coefficients=ones)
    hps.build_solver(pde)
    with pytest.raises(ValueError):
        hps.solve(pde, np.zeros(dom.boundary_points.shape[0]), source=ones)

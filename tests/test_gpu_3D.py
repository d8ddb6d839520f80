"""GPU parity of the 3D uniform DtN path (leaf solve, oct merges, down
pass) against the FP64 oracle, plus the 3D analytic case through the GPU.

Tolerances: FP64 path vs the FP64 oracle, relative max error <= 1e-11
(1e-10 for merge operators); analytic polynomial case <= 1e-10 absolute.
"""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300 import _stages as st
from jaxhps_gb300 import _stages_3D as st3
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _problem3(L, p, q, nsrc=None, seed=0, extra=False):
    rng = np.random.default_rng(seed)
    rb = (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=hps.DiscretizationNode3D(*rb), L=L)
    x = dom.interior_points
    c = 1.0 + 0.3 * np.exp(-((x[..., 0] - 0.2) ** 2 + (x[..., 1] + 0.3) ** 2 + x[..., 2] ** 2) / 0.1)
    ones = np.ones_like(c)
    f = rng.standard_normal(x.shape[:2] + ((nsrc,) if nsrc else ()))
    coeffs = {"D_xx": ones, "D_yy": ones, "D_zz": ones, "I": -c}
    kw = dict(D_xx_coefficients=ones, D_yy_coefficients=ones, D_zz_coefficients=ones, I_coefficients=-c)
    if extra:
        coeffs["D_xz"] = 0.1 * np.cos(x[..., 1])
        coeffs["D_y"] = 0.2 * x[..., 2]
        kw["D_xz_coefficients"] = coeffs["D_xz"]
        kw["D_y_coefficients"] = coeffs["D_y"]
    pde = hps.PDEProblem(dom, source=f, **kw)
    ref = O.Problem3D(rb, L, p, q, coeffs, f)
    return dom, pde, ref


@pytest.mark.parametrize("L,p,q,nsrc,extra", [(1, 6, 4, None, False), (1, 8, 6, 3, True)])
def test_leaf_stage_3D_matches_oracle(cuda, L, p, q, nsrc, extra):
    dom, pde, ref = _problem3(L, p, q, nsrc, extra=extra)
    Y, T, v, h = st.local_solve_stage_uniform_3D_DtN(pde, device=cuda)
    A = O.assemble_operator(ref.coeffs, ref.ops, dom.n_leaves, p ** 3)
    Yr, Tr, vr, hr = O.leaf_dtn(A, ref.source, ref.P, ref.Q)
    if nsrc is None:
        vr, hr = vr[..., 0], hr[..., 0]
    for a, b in ((Y, Yr), (T, Tr), (v, vr), (h, hr)):
        assert tuple(a.shape) == b.shape and _rel(a, b) < 1e-11


@pytest.mark.parametrize("L,p,q,nsrc,extra", [(1, 6, 4, None, False), (2, 6, 4, 2, True), (1, 10, 8, None, False)])
def test_build_solve_3D_matches_oracle(cuda, L, p, q, nsrc, extra):
    dom, pde, ref = _problem3(L, p, q, nsrc, seed=1, extra=extra)
    T_top = hps.build_solver(pde, return_top_T=True)
    bp = dom.boundary_points
    g = np.sin(bp[:, 0]) + bp[:, 1] * bp[:, 2]
    if nsrc:
        g = np.stack([g * (k + 1) for k in range(nsrc)], -1)
    u = hps.solve(pde, g)
    ref.build()
    ur = ref.solve(g)
    assert tuple(u.shape) == ur.shape
    assert _rel(u, ur) < 1e-11
    assert _rel(T_top, ref.T_top) < 1e-10
    assert len(pde.S_lst) == len(ref.S_lst)
    for a, b in zip(pde.S_lst, ref.S_lst):
        assert tuple(a.shape) == b.shape and _rel(a, b) < 1e-10
    assert pde.S_lst[-1].dim() == 2   # root stored without a batch axis, like the reference


def test_merge_stage_3D_without_top_T(cuda):
    """The top merged map is skipped unless asked for; S and g~ are unchanged."""
    dom, pde, ref = _problem3(2, 6, 4, 2, seed=3)
    Y, T, v, h = st.local_solve_stage_uniform_3D_DtN(pde, device=cuda)
    S1, g1 = st3.merge_stage_uniform_3D_DtN(T, h, l=2, device=cuda)
    S2, g2, Ttop = st3.merge_stage_uniform_3D_DtN(T, h, l=2, device=cuda, return_T=True)
    for a, b in zip(S1 + g1, S2 + g2):
        assert torch.equal(a, b)
    assert S1[-1].dim() == 2 and g1[-1].dim() == 2
    assert tuple(Ttop.shape) == (24 * 16 * 4, 24 * 16 * 4)


def test_polynomial_known_answer_3D_gpu(cuda):
    """u = x^3 - 3 x y^2 + z^2 with Laplacian 2, reproduced to rounding."""
    root = hps.DiscretizationNode3D(-1.0, 1.0, -0.5, 1.5, 0.0, 2.0)
    dom = hps.Domain(p=6, q=4, root=root, L=2)
    x = dom.interior_points
    ones = np.ones(x.shape[:2])
    pde = hps.PDEProblem(dom, source=2 * ones, D_xx_coefficients=ones, D_yy_coefficients=ones,
                         D_zz_coefficients=ones)
    hps.build_solver(pde)
    bp = dom.boundary_points
    u = hps.solve(pde, bp[:, 0] ** 3 - 3 * bp[:, 0] * bp[:, 1] ** 2 + bp[:, 2] ** 2).numpy()
    ue = x[..., 0] ** 3 - 3 * x[..., 0] * x[..., 1] ** 2 + x[..., 2] ** 2
    assert np.abs(u - ue).max() < 1e-10


def test_float32_build_3D_is_close(cuda):
    dom, pde, ref = _problem3(1, 8, 6, None, seed=5)
    hps.build_solver(pde, precision="float32")
    g = np.cos(dom.boundary_points[:, 0])
    u = hps.solve(pde, g)
    ur = ref.build().solve(g)
    assert _rel(u, ur) < 1e-3

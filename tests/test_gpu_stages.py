"""GPU parity of the HPS stages against the FP64 oracle (seeded inputs at
sizes the oracle finishes in seconds), plus the reference's analytic
known-answer case run end to end through the GPU path.

Tolerances: FP64 path vs the FP64 oracle, relative max error <= 1e-11
(both compute the same explicit inverses; only rounding differs).
"""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300 import _stages as st
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu

PI = np.pi


def _problem(L, p, q, nsrc=None, seed=0, root=(-1.0, 1.0, -1.0, 1.0), extra=False):
    rng = np.random.default_rng(seed)
    rootn = hps.DiscretizationNode2D(*root)
    dom = hps.Domain(p=p, q=q, root=rootn, L=L)
    x = dom.interior_points
    c = 1.0 + 0.5 * np.exp(-((x[..., 0] - 0.2) ** 2 + (x[..., 1] + 0.3) ** 2) / 0.04)
    ones = np.ones_like(c)
    shape = x.shape[:2] + ((nsrc,) if nsrc else ())
    f = rng.standard_normal(shape)
    coeffs = {"D_xx": ones, "D_yy": ones, "I": c}
    kw = dict(D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c)
    if extra:
        bx = 0.3 * np.sin(x[..., 1])
        coeffs["D_x"] = bx
        kw["D_x_coefficients"] = bx
    pde = hps.PDEProblem(dom, source=f, **kw)
    ref = O.Problem2D(root, L, p, q, coeffs, f)
    return dom, pde, ref


def _rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("L,p,q,nsrc", [(1, 6, 4, None), (2, 8, 6, 3), (1, 16, 14, None)])
def test_leaf_stage_matches_oracle(cuda, L, p, q, nsrc):
    dom, pde, ref = _problem(L, p, q, nsrc)
    Y, T, v, h = st.local_solve_stage_uniform_2D_DtN(pde, device=cuda)
    A = O.assemble_operator(ref.coeffs, ref.ops, dom.n_leaves, p * p)
    Yr, Tr, vr, hr = O.leaf_dtn(A, ref.source, ref.P, ref.Q)
    if nsrc is None:
        vr, hr = vr[..., 0], hr[..., 0]
    assert _rel(Y, Yr) < 1e-11
    assert _rel(T, Tr) < 1e-11
    assert _rel(v, vr) < 1e-11
    assert _rel(h, hr) < 1e-11


@pytest.mark.parametrize("L,p,q", [(1, 6, 4), (3, 8, 6)])
def test_merge_stage_matches_oracle(cuda, L, p, q):
    dom, pde, ref = _problem(L, p, q, 2, seed=1)
    Y, T, v, h = st.local_solve_stage_uniform_2D_DtN(pde, device=cuda)
    S_lst, g_lst, Ttop = st.merge_stage_uniform_2D_DtN(T, h, l=L, device=cuda, return_T=True)
    ref.build()
    assert len(S_lst) == len(ref.S_lst)
    for a, b in zip(S_lst, ref.S_lst):
        assert a.shape == b.shape and _rel(a, b) < 1e-10
    for a, b in zip(g_lst, ref.g_lst):
        assert _rel(a, b) < 1e-10
    assert _rel(Ttop, ref.T_top) < 1e-10


@pytest.mark.parametrize("L,p,q,nsrc,extra", [(2, 8, 6, None, False), (3, 8, 6, 4, True), (2, 12, 10, None, True)])
def test_build_solve_matches_oracle(cuda, L, p, q, nsrc, extra):
    dom, pde, ref = _problem(L, p, q, nsrc, seed=2, extra=extra)
    T_top = hps.build_solver(pde, return_top_T=True)
    bp = dom.boundary_points
    g = np.sin(bp[:, 0]) + bp[:, 1] ** 2
    if nsrc:
        g = np.stack([g * (k + 1) for k in range(nsrc)], -1)
    u = hps.solve(pde, g)
    ref.build()
    ur = ref.solve(g)
    assert tuple(u.shape) == ur.shape
    assert _rel(u, ur) < 1e-11
    assert _rel(T_top, ref.T_top) < 1e-10


@pytest.mark.parametrize("L,p,q", [(1, 6, 4), (2, 8, 6)])
def test_polynomial_known_answer_gpu(cuda, L, p, q):
    """tests/test_accuracy/test_single_merge_accuracy.py:56-166 through the GPU path."""
    root = hps.DiscretizationNode2D(-PI / 2, PI / 2, -PI / 2, PI / 2)
    dom = hps.Domain(p=p, q=q, root=root, L=L)
    x = dom.interior_points
    f = 2 * x[..., 1] * (x[..., 1] ** 2 - (PI / 2) ** 2) + 6 * x[..., 1] * (x[..., 0] ** 2 - (PI / 2) ** 2)
    ones = np.ones(x.shape[:2])
    pde = hps.PDEProblem(dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones)
    hps.build_solver(pde)
    bp = dom.boundary_points
    u = hps.solve(pde, bp[:, 0] ** 2 - bp[:, 1] ** 2).numpy()
    exact = x[..., 0] ** 2 - x[..., 1] ** 2 + x[..., 1] * (x[..., 1] ** 2 - (PI / 2) ** 2) * (
        x[..., 0] ** 2 - (PI / 2) ** 2)
    assert np.abs(u - exact).max() < 1e-12 * 10


def test_float32_build_is_close(cuda):
    dom, pde, ref = _problem(2, 8, 6, None, seed=4)
    hps.build_solver(pde, precision="float32")
    bp = dom.boundary_points
    g = np.cos(bp[:, 0])
    u = hps.solve(pde, g)
    ur = ref.build().solve(g)
    assert _rel(u, ur) < 1e-3


def _iti_problem(L, p, q, nsrc=None, seed=0, eta=4.0):
    rng = np.random.default_rng(seed)
    rootn = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=rootn, L=L)
    x = dom.interior_points
    k = 6.0
    qv = 0.5 * np.exp(-((x[..., 0] - 0.2) ** 2 + (x[..., 1] + 0.3) ** 2) / 0.05)
    ones = np.ones_like(qv)
    Icoef = k ** 2 * (1 + qv)
    shape = x.shape[:2] + ((nsrc,) if nsrc else ())
    f = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    pde = hps.PDEProblem(dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=Icoef,
                         use_ItI=True, eta=eta)
    ref = O.Problem2D(rootn.bounds, L, p, q, {"D_xx": ones, "D_yy": ones, "I": Icoef}, f, iti=True, eta=eta)
    return dom, pde, ref


@pytest.mark.parametrize("L,p,q,nsrc", [(1, 8, 6, None), (2, 10, 8, 3), (3, 8, 6, None)])
def test_iti_build_solve_matches_oracle(cuda, L, p, q, nsrc):
    dom, pde, ref = _iti_problem(L, p, q, nsrc)
    T_top = hps.build_solver(pde, return_top_T=True)
    bp = dom.boundary_points
    g = np.exp(1j * bp[:, 0]) + bp[:, 1]
    if nsrc:
        g = np.stack([g * (k + 1) for k in range(nsrc)], -1)
    u = hps.solve(pde, g)
    ref.build()
    ur = ref.solve(g)
    assert tuple(u.shape) == ur.shape
    assert _rel(u, ur) < 1e-11
    assert _rel(T_top, ref.T_top) < 1e-11
    for a, b in zip(pde.S_lst, ref.S_lst):
        assert _rel(a, b) < 1e-10


def test_iti_polynomial_known_answer_gpu(cuda):
    """ItI analytic case with complex coefficients (tests/test_accuracy/cases.py:212-265)
    through the GPU path: u = x^3 + 3y^2, (Delta + 1 + 0.1i) u = f."""
    PI2 = np.pi / 2
    root = hps.DiscretizationNode2D(-PI2, PI2, -PI2, PI2)
    L, p, q, eta = 2, 10, 8, 1.0
    dom = hps.Domain(p=p, q=q, root=root, L=L)
    x = dom.interior_points
    cc = 1.0 + 0.1j
    u_ex = x[..., 0] ** 3 + 3 * x[..., 1] ** 2
    f = 6 * x[..., 0] + 6 + cc * u_ex
    ones = np.ones(x.shape[:2])
    pde = hps.PDEProblem(dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=cc * ones,
                         use_ItI=True, eta=eta)
    hps.build_solver(pde)
    bp = dom.boundary_points
    n = bp.shape[0] // 4
    dn = np.concatenate([-6 * bp[:n, 1], 3 * bp[n:2 * n, 0] ** 2, 6 * bp[2 * n:3 * n, 1], -3 * bp[3 * n:, 0] ** 2])
    imp = dn + 1j * eta * (bp[:, 0] ** 3 + 3 * bp[:, 1] ** 2)
    u = hps.solve(pde, imp).numpy()
    assert np.abs(u - u_ex).max() < 1e-9


def _mixed_coefficients(x):
    """Every 2D operator kind, coefficients of different sizes and signs."""
    return {"D_xx": 1.0 + 0.3 * np.sin(x[..., 0]), "D_xy": 0.2 * np.cos(x[..., 1]),
            "D_yy": 1.5 + 0.1 * x[..., 0] * x[..., 1], "D_x": 3.0 * x[..., 1], "D_y": -2.0 * np.exp(x[..., 0]),
            "I": -(50.0 + 20.0 * np.sin(2.0 * x[..., 1]))}


def test_float32_leaf_operators_match_oracle(cuda):
    """FP32 leaf solve, its operator rows assembled in double-float
    arithmetic on the FP32 pipe: Y, T and the leaf inverse against the FP64
    oracle to FP32-level accuracy, every operator kind."""
    L, p, q = 2, 10, 8
    rootn = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=rootn, L=L)
    coeffs = _mixed_coefficients(dom.interior_points)
    pde = hps.PDEProblem(dom, **{f"{k}_coefficients": v for k, v in coeffs.items()})
    Y, T, _, _, Aii = st._local_solve_dtn(pde, pde.P, pde.Q, cuda, torch.float32, keep_inverse=True,
                                          want_source=False)
    ref = O.Problem2D(rootn.bounds, L, p, q, coeffs, np.zeros(dom.interior_points.shape[:2]))
    A = O.assemble_operator(ref.coeffs, ref.ops, dom.n_leaves, p * p)
    Yr, Tr, _, _ = O.leaf_dtn(A, np.zeros((dom.n_leaves, p * p, 1)), ref.P, ref.Q)
    # NumPy's float32 inverse of the same matrices: 1e-7 .. 2e-7 relative
    assert _rel(Y, Yr) < 1e-5
    assert _rel(T, Tr) < 1e-5
    ncb = 4 * (p - 1)
    eye = np.eye(p * p - ncb)
    prod = np.einsum("lij,ljk->lik", Aii.double().cpu().numpy(), A[:, ncb:, ncb:])
    assert np.abs(prod - eye).max() < 1e-5


def test_complex64_iti_leaf_operators_match_oracle(cuda):
    """complex64 ItI leaf solve with real coefficients (operator rows in
    double-float, as the FP32 build): Y and T against the complex128 oracle."""
    L, p, q, eta = 2, 10, 8, 6.0
    rootn = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=rootn, L=L)
    x = dom.interior_points
    coeffs = _mixed_coefficients(x)
    coeffs["I"] = 36.0 * (1.0 + 0.3 * np.exp(-(x ** 2).sum(-1)))
    rng = np.random.default_rng(3)
    f = rng.standard_normal(x.shape[:2]) + 1j * rng.standard_normal(x.shape[:2])
    pde = hps.PDEProblem(dom, source=f, use_ItI=True, eta=eta, **{f"{k}_coefficients": v for k, v in coeffs.items()})
    Y, T, v, h = st.local_solve_stage_uniform_2D_ItI(pde, device=cuda, dtype=torch.complex64)
    ref = O.Problem2D(rootn.bounds, L, p, q, coeffs, f, iti=True, eta=eta)
    A = O.assemble_operator(ref.coeffs, ref.ops, dom.n_leaves, p * p)
    Yr, Tr, vr, hr = O.leaf_iti(A, ref.source, ref.P, ref.QH, ref.G)
    # NumPy's complex64 inverse of the same matrices (condition ~5e3): 5e-7 .. 8e-7
    assert _rel(Y, Yr) < 3e-5
    assert _rel(T, Tr) < 3e-5
    assert _rel(v, vr[..., 0]) < 3e-5

"""GPU tests of the recursive 2 x 2 block inversion of the FP32 merge
interface matrices (hps_inverse_block_policy): the FP32 merge operators it
produces against the FP64 build and against the pivoted Gauss-Jordan path,
and the mixed-precision solve with it against the FP64 oracle.

Tolerances: FP32 operators relative max error against FP64 within 4x the
pivoted path's own error (plus 1e-6); the refined solution <= 1e-10 relative
to the oracle, as for every mixed-precision test."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300 import _native as nat
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


def _problem(L, p, q, nsrc=2, seed=0):
    """nsrc None: one right-hand side without the trailing axis."""
    rng = np.random.default_rng(seed)
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=root, L=L)
    x = dom.interior_points
    c = 1.0 + 0.5 * np.exp(-((x[..., 0] - 0.3) ** 2 + (x[..., 1] + 0.2) ** 2) / 0.04)
    ones = np.ones_like(c)
    f = rng.standard_normal(x.shape[:2] + ((nsrc,) if nsrc else ()))
    kw = dict(D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c)
    ref = O.Problem2D(root.bounds, L, p, q, {"D_xx": ones, "D_yy": ones, "I": c}, f)
    return dom, f, kw, ref


def _build(dom, f, kw, precision, policy):
    old = nat.lib().hps_inverse_block_policy(policy)
    try:
        pde = hps.PDEProblem(dom, source=f, **kw)
        hps.build_solver(pde, precision=precision)
        torch.cuda.synchronize()
    finally:
        nat.lib().hps_inverse_block_policy(old)
    return pde


def _rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_block_inverse_merge_operators_match_fp64(cuda):
    """L = 4, p = 16: interface matrices of n = 56, 112, 224, 448; the last two
    are inverted by the block recursion in FP32."""
    dom, f, kw, _ = _problem(4, 16, 14)
    p64 = _build(dom, f, kw, "float64", 1)
    p_blk = _build(dom, f, kw, "float32", 1)
    p_piv = _build(dom, f, kw, "float32", 0)
    for lvl in (2, 3):
        S64 = p64.S_lst[lvl].cpu().numpy()
        e_blk = _rel(p_blk.S_lst[lvl].cpu().numpy(), S64)
        e_piv = _rel(p_piv.S_lst[lvl].cpu().numpy(), S64)
        assert e_blk <= 4 * e_piv + 1e-6, (lvl, e_blk, e_piv)
        assert e_blk < 1e-3, (lvl, e_blk)


@pytest.mark.parametrize("L,nsrc", [(4, 3), (5, None)])
def test_mixed_solve_with_block_inverse_matches_oracle(cuda, L, nsrc):
    dom, f, kw, ref = _problem(L, 16, 14, nsrc=nsrc, seed=L)
    bp = dom.boundary_points
    g = np.sin(bp[:, 0]) + bp[:, 1] ** 2
    if nsrc:
        g = np.stack([g * (k + 1) for k in range(nsrc)], -1)
    hist = {}
    sols = {}
    for policy in (1, 0):
        pde = _build(dom, f, kw, "mixed", policy)
        sols[policy] = hps.solve(pde, g).numpy()
        hist[policy] = list(pde._state.history)
    ur = ref.build().solve(g)
    for policy in (1, 0):
        assert _rel(sols[policy], ur) < 1e-10, (policy, hist[policy])
    assert len(hist[1]) <= len(hist[0]) + 1, hist


@pytest.mark.parametrize("n,batch", [(56, 5), (100, 3), (112, 300), (128, 2), (224, 3), (448, 2), (900, 1)])
def test_interface_inverse_matches_numpy(cuda, n, batch):
    """The block recursion on diagonally dominant matrices (no row
    permutation: pivots stay within blocks), out of place and in place."""
    rng = np.random.default_rng(n)
    A = (rng.standard_normal((batch, n, n)) + 2 * np.sqrt(n) * np.eye(n)).astype(np.float32)
    tA = torch.as_tensor(A, device=cuda)
    info = torch.full((batch,), -7, dtype=torch.int32, device=cuda)
    old = nat.lib().hps_inverse_block_policy(1)
    try:
        X = nat.inverse(tA, info=info, entry="hps_inverse_interface").cpu().numpy()
        nat.inverse(tA, out=tA, entry="hps_inverse_interface")
    finally:
        nat.lib().hps_inverse_block_policy(old)
    assert (info.cpu().numpy() == 0).all()
    Xe = np.linalg.inv(A.astype(np.float64))
    assert _rel(X, Xe) < 2e-5 * 20
    assert np.array_equal(tA.cpu().numpy(), X)


@pytest.mark.parametrize("n,col", [(112, 37), (448, 300)])
def test_block_inverse_reports_a_singular_interface_block_at_its_column(cuda, n, col):
    """A zero column: info > 0 for that matrix only, the other inverted exactly."""
    D = torch.eye(n, dtype=torch.float32, device=cuda).repeat(2, 1, 1).contiguous()
    D[1, :, col] = 0.0
    info = torch.zeros(2, dtype=torch.int32, device=cuda)
    old = nat.lib().hps_inverse_block_policy(1)
    try:
        X = nat.inverse(D, info=info, entry="hps_inverse_interface")
    finally:
        nat.lib().hps_inverse_block_policy(old)
    inf = info.cpu().numpy()
    assert inf[0] == 0 and inf[1] > 0
    assert torch.equal(X[0], torch.eye(n, dtype=torch.float32, device=cuda))


def test_block_inverse_reports_a_singular_interface_block(cuda):
    """A zero interface matrix block makes the recursion report a zero pivot
    (info > 0) instead of returning silently, like the pivoted path."""
    n, nm = 448, 2
    D = torch.eye(n, dtype=torch.float32, device=cuda).repeat(nm, 1, 1).contiguous()
    D[1, :, 300] = 0.0   # singular in the Schur-complement half
    info = torch.zeros(nm, dtype=torch.int32, device=cuda)
    old = nat.lib().hps_inverse_block_policy(1)
    try:
        X = nat.inverse(D, info=info, entry="hps_inverse_interface")
    finally:
        nat.lib().hps_inverse_block_policy(old)
    inf = info.cpu().numpy()
    assert inf[0] == 0 and inf[1] > 0
    assert torch.equal(X[0], torch.eye(n, dtype=torch.float32, device=cuda))

"""GPU tests of mixed precision: the FP64 residual kernel against dense
NumPy, and FP32-build + FP64-residual refinement against the FP64 oracle.

Tolerance for the refined solution: relative max error <= 1e-10 against the
FP64 oracle (the target stated for the mixed path)."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300 import _refinement as rf
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


def _setup(L, p, q, nsrc, extra, seed=0):
    rng = np.random.default_rng(seed)
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=root, L=L)
    x = dom.interior_points
    c = 1.0 + 0.5 * np.exp(-((x[..., 0] - 0.2) ** 2 + (x[..., 1] + 0.3) ** 2) / 0.04)
    ones = np.ones_like(c)
    coeffs = {"D_xx": ones, "D_yy": ones, "I": c}
    kw = dict(D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c)
    if extra:
        bx = 0.3 * np.sin(x[..., 1])
        bxy = 0.2 * np.cos(x[..., 0])
        coeffs.update({"D_x": bx, "D_xy": bxy})
        kw.update(D_x_coefficients=bx, D_xy_coefficients=bxy)
    shape = x.shape[:2] + ((nsrc,) if nsrc else ())
    f = rng.standard_normal(shape)
    return dom, hps.PDEProblem(dom, source=f, **kw), O.Problem2D(root.bounds, L, p, q, coeffs, f)


@pytest.mark.parametrize("extra", [False, True])
def test_residual_kernel_matches_dense(cuda, extra):
    L, p, q, ns = 2, 8, 6, 3
    dom, pde, ref = _setup(L, p, q, ns, extra)
    hps.build_solver(pde, precision="mixed")
    state = pde._state
    rng = np.random.default_rng(1)
    nl, ncb = dom.n_leaves, 4 * (p - 1)
    u_int = rng.standard_normal((nl, p * p - ncb, ns))
    g = rng.standard_normal((nl, 4 * q, ns))
    tu = torch.as_tensor(u_int, device=cuda)
    tg = torch.as_tensor(g, device=cuda)
    r32 = torch.empty(u_int.shape, dtype=torch.float32, device=cuda)
    flux = torch.empty(g.shape, dtype=torch.float64, device=cuda)
    ufull = torch.empty((nl, p * p, ns), dtype=torch.float64, device=cuda)
    rf._residual(state, tu, tg, r32, flux, u_full=ufull)
    A = O.assemble_operator(ref.coeffs, ref.ops, nl, p * p)
    full = np.concatenate([np.einsum("ij,ljs->lis", ref.P, g), u_int], axis=1)
    r_ref = ref.source[:, ncb:] - np.einsum("lij,ljs->lis", A[:, ncb:, :], full)
    F_ref = np.einsum("ij,ljs->lis", ref.Q, full)
    assert np.allclose(ufull.cpu().numpy(), full, atol=1e-12)
    scale = np.abs(r_ref).max()
    assert np.abs(r32.cpu().numpy() - r_ref).max() < 1e-6 * scale
    assert np.abs(flux.cpu().numpy() - F_ref).max() < 1e-11 * np.abs(F_ref).max()


@pytest.mark.parametrize("L,p,q,nsrc,extra", [(2, 8, 6, None, False), (3, 12, 10, 4, True), (3, 16, 14, 2, False)])
def test_mixed_matches_fp64_oracle(cuda, L, p, q, nsrc, extra):
    dom, pde, ref = _setup(L, p, q, nsrc, extra, seed=2)
    hps.build_solver(pde, precision="mixed")
    bp = dom.boundary_points
    g = np.sin(bp[:, 0]) + bp[:, 1] ** 2
    if nsrc:
        g = np.stack([g * (k + 1) for k in range(nsrc)], -1)
    u = hps.solve(pde, g).numpy()
    ur = ref.build().solve(g)
    assert u.shape == ur.shape
    err = np.abs(u - ur).max() / np.abs(ur).max()
    hist = pde._state.history
    assert err < 1e-10, (err, hist)
    assert len(hist) < pde._state.max_iters

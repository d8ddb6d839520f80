"""GPU tests of the dimension-generic mixed-precision path (FP32 HPS build
refined against FP64 residuals from the assembled interior rows): 3D
against the FP64 oracle, 2D against the oracle and the tensor-product
path, and 3D at the full c4 size (512 leaves, p = 10) against the plain
FP64 GPU path.  Tolerance: relative max error <= 1e-10."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300 import _refinement_dense as rd
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _problem3(L, p, q, nsrc, seed=0):
    rng = np.random.default_rng(seed)
    rb = (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=hps.DiscretizationNode3D(*rb), L=L)
    x = dom.interior_points
    c = 1.0 + 0.3 * np.exp(-((x[..., 0] - 0.2) ** 2 + (x[..., 1] + 0.3) ** 2 + x[..., 2] ** 2) / 0.1)
    ones = np.ones_like(c)
    f = rng.standard_normal(x.shape[:2] + ((nsrc,) if nsrc else ()))
    kw = dict(D_xx_coefficients=ones, D_yy_coefficients=ones, D_zz_coefficients=ones, I_coefficients=c,
              D_z_coefficients=0.2 * x[..., 0])
    coeffs = {"D_xx": ones, "D_yy": ones, "D_zz": ones, "I": c, "D_z": 0.2 * x[..., 0]}
    return dom, hps.PDEProblem(dom, source=f, **kw), O.Problem3D(rb, L, p, q, coeffs, f)


@pytest.mark.parametrize("L,p,q,nsrc", [(1, 8, 6, None), (2, 6, 4, 3)])
def test_mixed_3D_matches_oracle(cuda, L, p, q, nsrc):
    dom, pde, ref = _problem3(L, p, q, nsrc)
    hps.build_solver(pde, precision="mixed")
    bp = dom.boundary_points
    g = np.cos(bp[:, 0]) + bp[:, 1] * bp[:, 2]
    if nsrc:
        g = np.stack([g * (k + 1) for k in range(nsrc)], -1)
    u = hps.solve(pde, g)
    ur = ref.build().solve(g)
    assert tuple(u.shape) == ur.shape
    assert _rel(u, ur) < 1e-10
    assert len(pde._state.history) <= 12


def test_dense_mixed_path_2D_matches_oracle_and_tensor_path(cuda):
    rng = np.random.default_rng(2)
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    L, p, q = 3, 10, 8
    dom = hps.Domain(p=p, q=q, root=root, L=L)
    x = dom.interior_points
    c = 1.0 + 0.5 * np.exp(-((x[..., 0] - 0.2) ** 2 + (x[..., 1] + 0.3) ** 2) / 0.04)
    ones = np.ones_like(c)
    f = rng.standard_normal(x.shape[:2] + (2,))
    kw = dict(D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c)
    g = np.stack([dom.boundary_points[:, 0] ** 2, np.sin(dom.boundary_points[:, 1])], -1)
    ur = O.Problem2D(root.bounds, L, p, q, {"D_xx": ones, "D_yy": ones, "I": c}, f).build().solve(g)
    pde = hps.PDEProblem(dom, source=f, **kw)
    rd.build_mixed_dense(pde)
    u_dense = rd.solve_mixed_dense(pde, g)
    assert _rel(u_dense, ur) < 1e-10
    pde2 = hps.PDEProblem(dom, source=f, **kw)
    hps.build_solver(pde2, precision="mixed")
    u_tensor = hps.solve(pde2, g)
    assert _rel(u_tensor, ur) < 1e-10


def test_mixed_3D_full_size_matches_fp64_path(cuda):
    """c4 sizes: 512 leaves, p = 10, q = 8, variable zeroth-order coefficient;
    manufactured u = sin(pi x) sin(pi y) sin(pi z)."""
    L, p, q = 3, 10, 8
    dom = hps.Domain(p=p, q=q, root=hps.DiscretizationNode3D(-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), L=L)
    x = dom.interior_points
    rng = np.random.default_rng(3)
    z = rng.uniform(-0.8, 0.8, (6, 3))
    c = 1 + 0.3 * sum(np.exp(-((x - zk) ** 2).sum(-1) / 0.04) for zk in z)
    u_ex = np.sin(np.pi * x[..., 0]) * np.sin(np.pi * x[..., 1]) * np.sin(np.pi * x[..., 2])
    f = (-3 * np.pi ** 2 + c) * u_ex
    ones = np.ones_like(c)
    kw = dict(D_xx_coefficients=ones, D_yy_coefficients=ones, D_zz_coefficients=ones, I_coefficients=c)
    g = np.zeros(dom.boundary_points.shape[0])
    pde64 = hps.PDEProblem(dom, source=f, **kw)
    hps.build_solver(pde64)
    u64 = hps.solve(pde64, g).numpy()
    del pde64
    torch.cuda.empty_cache()
    pde = hps.PDEProblem(dom, source=f, **kw)
    hps.build_solver(pde, precision="mixed")
    u = hps.solve(pde, g).numpy()
    assert _rel(u, u64) < 1e-10
    assert np.abs(u - u_ex).max() < 1e-7      # discretisation error of p = 10

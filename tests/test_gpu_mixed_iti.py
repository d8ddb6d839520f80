"""Mixed-precision ItI: complex64 HPS build refined against complex128
residuals, against the complex128 oracle (relative max error <= 1e-10)."""

import numpy as np
import pytest

import jaxhps_gb300 as hps
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = a.numpy() if hasattr(a, "numpy") else np.asarray(a)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("L,p,q,k,nsrc", [(2, 10, 8, 10.0, None), (3, 12, 10, 20.0, 2)])
def test_mixed_iti_matches_oracle(cuda, L, p, q, k, nsrc):
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=root, L=L)
    x = dom.interior_points
    rng = np.random.default_rng(int(k))
    z = rng.uniform(-0.8, 0.8, (6, 2))
    qv = 0.5 * sum(np.exp(-((x - zk) ** 2).sum(-1) / 0.05 ** 2 * 0.25) for zk in z)
    Icoef = k ** 2 * (1 + qv)
    ones = np.ones_like(Icoef)
    shape = x.shape[:2] + ((nsrc,) if nsrc else ())
    f = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    pde = hps.PDEProblem(dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=Icoef,
                         use_ItI=True, eta=k)
    hps.build_solver(pde, precision="mixed")
    g = np.exp(1j * k * dom.boundary_points[:, 0] * 0.3)
    if nsrc:
        g = np.stack([g * (j + 1) for j in range(nsrc)], -1)
    u = hps.solve(pde, g)
    ur = O.Problem2D(root.bounds, L, p, q, {"D_xx": ones, "D_yy": ones, "I": Icoef}, f, iti=True, eta=k).build().solve(g)
    assert u.shape == ur.shape
    assert _rel(u, ur) < 1e-10
    assert len(pde._state.history) <= 15


def test_mixed_iti_helmholtz_scattering_vs_complex128(cuda):
    """The scattering workload (k=40, 20 Gaussian bumps of amplitude 0.5 and
    width 0.05, plane wave at a seeded angle, eta=k, p=16) at L=6: the
    refined complex64 solve against the complex128 solve, rel <= 1e-10, in
    at most 8 refinement steps."""
    p, q, k, L = 16, 14, 40.0, 6
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=root, L=L)
    x = dom.interior_points
    rng = np.random.default_rng(40)
    z = rng.uniform(-0.8, 0.8, (20, 2))
    qv = 0.5 * sum(np.exp(-((x - zk) ** 2).sum(-1) / (2 * 0.05 ** 2)) for zk in z)
    th = rng.uniform(0, 2 * np.pi)
    uin = np.exp(1j * k * (x @ np.array([np.cos(th), np.sin(th)])))
    ones = np.ones_like(qv)
    g = np.zeros(dom.boundary_points.shape[0], dtype=np.complex128)
    sols = {}
    for prec in ("float64", "mixed"):
        pde = hps.PDEProblem(dom, source=-k ** 2 * qv * uin, D_xx_coefficients=ones, D_yy_coefficients=ones,
                             I_coefficients=k ** 2 * (1 + qv), use_ItI=True, eta=k)
        hps.build_solver(pde, precision=prec)
        sols[prec] = hps.solve(pde, g).numpy()
        if prec == "mixed":
            assert len(pde._state.history) <= 8
        del pde
    assert _rel(sols["mixed"], sols["float64"]) < 1e-10


def test_mixed_iti_pinned_source_matches_numpy_source(cuda):
    """A page-locked complex128 source (copied while the build runs) gives
    the same solution, bit for bit, as the NumPy source."""
    import torch
    L, p, q, k = 3, 12, 10, 15.0
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=root, L=L)
    x = dom.interior_points
    rng = np.random.default_rng(7)
    Icoef = k ** 2 * (1 + 0.3 * np.exp(-(x ** 2).sum(-1) / 0.1))
    ones = np.ones_like(Icoef)
    f = rng.standard_normal(x.shape[:2] + (2,)) + 1j * rng.standard_normal(x.shape[:2] + (2,))
    g = np.exp(1j * k * dom.boundary_points[:, 1] * 0.4)
    sols = []
    for src in (f, torch.as_tensor(f).pin_memory()):
        pde = hps.PDEProblem(dom, source=src, D_xx_coefficients=ones, D_yy_coefficients=ones,
                             I_coefficients=Icoef, use_ItI=True, eta=k)
        hps.build_solver(pde, precision="mixed")
        sols.append(hps.solve(pde, g).numpy())
    assert np.array_equal(sols[0], sols[1])

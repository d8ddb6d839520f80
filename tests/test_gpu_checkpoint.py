"""GPU round trip of the operator-set save/load: build, save, load onto a
fresh problem over an equal domain, solve without a build; the solution is
bitwise the solution of the problem that was built (the same kernels run on
the same operators).  2D DtN in FP64 and mixed precision, 3D DtN mixed."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps

pytestmark = pytest.mark.gpu


def _pde2(L, p, q, nsrc, seed):
    rng = np.random.default_rng(seed)
    dom = hps.Domain(p=p, q=q, root=hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0), L=L)
    x = dom.interior_points
    c = 1.0 + 0.5 * np.exp(-((x[..., 0] - 0.2) ** 2 + (x[..., 1] + 0.3) ** 2) / 0.04)
    ones = np.ones_like(c)
    f = rng.standard_normal(x.shape[:2] + (nsrc,))
    return hps.PDEProblem(dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c)


def _pde3(L, p, q, nsrc, seed):
    rng = np.random.default_rng(seed)
    dom = hps.Domain(p=p, q=q, root=hps.DiscretizationNode3D(-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), L=L)
    x = dom.interior_points
    ones = np.ones(x.shape[:2])
    f = rng.standard_normal(x.shape[:2] + (nsrc,))
    return hps.PDEProblem(dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones, D_zz_coefficients=ones,
                          I_coefficients=1.0 + 0.1 * x[..., 0] ** 2)


@pytest.mark.parametrize("make,L,p,q,precision", [(_pde2, 3, 8, 6, "float64"), (_pde2, 3, 16, 14, "mixed"),
                                                  (_pde3, 1, 6, 4, "mixed")])
def test_loaded_operator_set_solves_bitwise(cuda, tmp_path, make, L, p, q, precision):
    built = make(L, p, q, 2, seed=L + p)
    hps.build_solver(built, precision=precision)
    path = tmp_path / "ops.pt"
    hps.save_solver(built, path)
    fresh = make(L, p, q, 2, seed=L + p)
    hps.load_solver(fresh, path, device=cuda)
    bp = built.domain.boundary_points
    g = np.stack([np.sin(bp[:, 0]) + k * bp[:, 1] ** 2 for k in range(2)], -1)
    u_built = hps.solve(built, g)
    u_loaded = hps.solve(fresh, g)
    assert torch.equal(u_built, u_loaded)
    assert np.isfinite(u_loaded.numpy()).all()

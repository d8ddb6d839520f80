"""The leaf stage in chunks of leaves (taken when the assembled leaf
operators of all leaves would exceed the workspace budget) gives the
unchunked result: every output of the FP64 leaf stage to 1e-13 relative."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300 import _stages as st

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim", [2, 3])
def test_chunked_leaf_stage_matches(cuda, dim, monkeypatch):
    if dim == 2:
        dom = hps.Domain(p=10, q=8, root=hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0), L=3)
    else:
        dom = hps.Domain(p=6, q=4, root=hps.DiscretizationNode3D(-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), L=2)
    x = dom.interior_points
    rng = np.random.default_rng(dim)
    ones = np.ones(x.shape[:2])
    kw = dict(D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=1.0 + x[..., 0] ** 2)
    if dim == 3:
        kw["D_zz_coefficients"] = ones
    pde = hps.PDEProblem(dom, source=rng.standard_normal(x.shape[:2] + (3,)), **kw)
    full = st._local_solve_dtn(pde, pde.P, pde.Q, cuda, torch.float64, True)
    monkeypatch.setattr(st, "LEAF_WORKSPACE_BUDGET", 1 << 16)   # a few leaves per chunk
    chunked = st._local_solve_dtn(pde, pde.P, pde.Q, cuda, torch.float64, True)
    for a, b in zip(full, chunked):
        assert float((a - b).abs().max() / a.abs().max()) < 1e-13

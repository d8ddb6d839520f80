"""The GEMM autotuner: shape recording, every kernel variant computing the
same product (against an FP64 torch product, FP32-level tolerance 1e-5
relative), the tuned table steering dispatch, and a tuned mixed-precision
build + solve matching the untuned one to 1e-10 relative."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300 import _native as nat
from jaxhps_gb300 import autotune as at

pytestmark = pytest.mark.gpu


def _problem(L=3, p=10, q=8, nsrc=4):
    dom = hps.Domain(p=p, q=q, root=hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0), L=L)
    x = dom.interior_points
    rng = np.random.default_rng(5)
    c = 1.0 + 0.5 * np.exp(-((x[..., 0] - 0.2) ** 2 + x[..., 1] ** 2) / 0.1)
    ones = np.ones_like(c)
    f = rng.standard_normal(x.shape[:2] + (nsrc,))
    g = np.stack([dom.boundary_points[:, 0] ** 2 * (k + 1) for k in range(nsrc)], -1)
    return dom, dict(source=f, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c), g


@pytest.mark.parametrize("M,N,K,batch", [(196, 64, 196, 40), (56, 64, 196, 17), (448, 448, 300, 2),
                                         (100, 24, 9, 3)])
def test_every_variant_computes_the_product(cuda, M, N, K, batch):
    g = torch.Generator(device=cuda).manual_seed(M + N)
    A = torch.randn(batch, M, K, device=cuda, generator=g)
    B = torch.randn(batch, K, N, device=cuda, generator=g)
    Cm = torch.randn(batch, M, N, device=cuda, generator=g)
    ref = (A.double() @ B.double()) * 0.5 + Cm.double() * 2.0
    lib = nat.lib()
    try:
        for v in at.VARIANTS:
            lib.hps_gemm_force_variant(v)
            D = torch.full((batch, M, N), float("nan"), device=cuda)
            nat.gemm(A, B, D, alpha=0.5, beta=2.0, Cmat=Cm)
            torch.cuda.synchronize()
            err = float((D.double() - ref).abs().max() / ref.abs().max())
            assert err < 1e-5, (v, err)
    finally:
        lib.hps_gemm_force_variant(-1)


def test_record_tune_and_apply(cuda):
    dom, kw, g = _problem()

    def run():
        pde = hps.PDEProblem(dom, **kw)
        hps.build_solver(pde, precision="mixed")
        return hps.solve(pde, g, host_device=None)

    u0 = run().cpu().numpy()
    shapes = at.record_shapes(run)
    assert len(shapes) >= 5 and all(len(s) == 13 for s in shapes)
    try:
        rep = at.tune(run, reps=2)
        assert len(rep["shapes"]) == len(shapes)
        assert all(s["ms"] <= s["builtin_ms"] * 1.5 for s in rep["shapes"])
        u1 = run().cpu().numpy()
        assert np.abs(u1 - u0).max() <= 1e-10 * np.abs(u0).max()
        # a stored variant is what runs: force-free dispatch of a tuned shape
        M, N, K, b = rep["shapes"][0]["M"], rep["shapes"][0]["N"], rep["shapes"][0]["K"], rep["shapes"][0]["batch"]
        assert nat.lib().hps_gemm_tune_set(M, N, K, b, 99) != 0
    finally:
        at.clear()
    assert nat.lib().hps_gemm_force_variant(-1) == -1

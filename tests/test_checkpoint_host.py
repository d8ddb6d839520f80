"""Operator-set save/load on the CPU: a round trip of a hand-made operator
set (tensors, the refinement state's dataclass, lists), the domain check,
and the refusals (unbuilt problem, adaptive tree).  The GPU round trip
through a real build is in test_gpu_checkpoint.py."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300._refinement import MixedState


def _pde(L=2, p=6, q=4, root=(-1.0, 1.0, -1.0, 1.0)):
    dom = hps.Domain(p=p, q=q, root=hps.DiscretizationNode2D(*root), L=L)
    ones = np.ones(dom.interior_points.shape[:2])
    return hps.PDEProblem(dom, source=ones, D_xx_coefficients=ones, D_yy_coefficients=ones)


def _fake_build(pde, seed=0):
    g = torch.Generator().manual_seed(seed)
    n = pde.domain.n_leaves
    pde.Y = torch.randn(n, 36, 16, generator=g, dtype=torch.float64)
    pde.v = torch.randn(n, 36, generator=g, dtype=torch.float64)
    pde.S_lst = [torch.randn(4, 8, 16, generator=g), torch.randn(1, 16, 32, generator=g)]
    pde.g_tilde_lst = [torch.randn(4, 8, generator=g)]
    pde._precision = "mixed"
    pde._state = MixedState(
        mixed=True, n_leaves=n, p=6, q=4, Y_int=pde.Y[:, 20:, :].float(), Aii_inv=torch.randn(n, 16, 16, generator=g),
        Q_int=torch.randn(16, 16, generator=g), S_lst=pde.S_lst, Dinv_lst=[torch.randn(4, 8, 8, generator=g)],
        B_lst=[torch.randn(4, 16, 8, generator=g)], coeffs=torch.randn(2, n, 36, generator=g, dtype=torch.float64),
        op_kind=[0, 1], f=torch.randn(n, 36, 1, generator=g, dtype=torch.float64), multi=False,
        consts={"D1": torch.randn(6, 6, generator=g, dtype=torch.float64)}, nbr=torch.arange(10, dtype=torch.int32),
        bnode=torch.arange(5, dtype=torch.int32), history=[1.0, 1e-3])
    return pde


def test_round_trip_restores_every_tensor(tmp_path):
    src = _fake_build(_pde())
    path = tmp_path / "ops.pt"
    hps.save_solver(src, path)
    dst = _pde()
    hps.load_solver(dst, path, device="cpu")
    assert dst._precision == "mixed"
    assert torch.equal(dst.Y, src.Y) and torch.equal(dst.v, src.v)
    assert len(dst.S_lst) == 2 and all(torch.equal(a, b) for a, b in zip(dst.S_lst, src.S_lst))
    assert torch.equal(dst.g_tilde_lst[0], src.g_tilde_lst[0])
    a, b = dst._state, src._state
    assert isinstance(a, MixedState) and a.op_kind == b.op_kind and a.history == b.history
    for name in ("Y_int", "Aii_inv", "Q_int", "coeffs", "f", "nbr", "bnode"):
        assert torch.equal(getattr(a, name), getattr(b, name)), name
    assert torch.equal(a.consts["D1"], b.consts["D1"])
    assert torch.equal(a.Dinv_lst[0], b.Dinv_lst[0]) and torch.equal(a.B_lst[0], b.B_lst[0])


@pytest.mark.parametrize("kw", [dict(L=3), dict(p=8, q=6), dict(root=(0.0, 1.0, 0.0, 1.0))])
def test_load_refuses_another_domain(tmp_path, kw):
    path = tmp_path / "ops.pt"
    hps.save_solver(_fake_build(_pde()), path)
    other = _pde(**kw)
    with pytest.raises(ValueError, match="another domain"):
        hps.load_solver(other, path, device="cpu")
    assert other._state is None and other.Y is None


def test_save_refuses_unbuilt_problem_and_load_refuses_other_files(tmp_path):
    with pytest.raises(ValueError, match="nothing to save"):
        hps.save_solver(_pde(), tmp_path / "x.pt")
    torch.save({"something": 1}, tmp_path / "y.pt")
    with pytest.raises(ValueError, match="not an operator set"):
        hps.load_solver(_pde(), tmp_path / "y.pt", device="cpu")


def test_adaptive_domains_are_refused(tmp_path):
    root = hps.DiscretizationNode2D(0.0, 1.0, 0.0, 1.0)
    dom = hps.Domain(p=6, q=4, root=root)
    ones = np.ones(dom.interior_points.shape[:2])
    pde = hps.PDEProblem(dom, source=ones, D_xx_coefficients=ones, D_yy_coefficients=ones)
    with pytest.raises(NotImplementedError):
        hps.save_solver(pde, tmp_path / "z.pt")

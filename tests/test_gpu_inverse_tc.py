"""The FP32 batched inverse whose Gauss-Jordan tableau lives in tensor memory
(tcgen05 trailing updates on three-part TF32 operands), through the C ABI:
hps_inverse_batched at hps_inverse_policy(2) against numpy.linalg.inv in FP64
and against the SIMT kernels (hps_inverse_policy(0)), on sizes across one and
two 128-row halves, strided inputs, a singular matrix, the leaf blocks of a
small-leaf operator, and the default policy (leaf stage only).

Tolerance: relative max error <= 2e-5 x cond-like growth for these
diagonally weighted random matrices (the SIMT FP32 inverse tests use 2e-5).
"""

import numpy as np
import pytest
import torch

from jaxhps_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def _mats(rng, batch, n):
    A = rng.standard_normal((batch, n, n)) + 2 * np.sqrt(n) * np.eye(n)
    return np.ascontiguousarray(A[:, rng.permutation(n), :])   # pivoting must reorder rows


@pytest.fixture
def policy():
    """Policy 2: hps_inverse_batched itself runs the tensor-memory kernel."""
    lib = nat.load_library()
    old = lib.hps_inverse_policy(2)
    yield lib
    lib.hps_inverse_policy(old)


@pytest.mark.parametrize("n,batch", [(65, 3), (100, 7), (128, 5), (129, 4), (196, 300), (200, 2), (224, 3)])
def test_tc_inverse_matches_numpy(cuda, policy, n, batch):
    rng = np.random.default_rng(n)
    A = _mats(rng, batch, n)
    At = torch.as_tensor(A, dtype=torch.float32, device=cuda)
    info = torch.full((batch,), -7, dtype=torch.int32, device=cuda)
    launches = nat.launch_count()
    X = nat.inverse(At, info=info)
    torch.cuda.synchronize()
    assert nat.launch_count() - launches == 1            # one launch: the tensor-memory kernel
    assert (info.cpu().numpy() == 0).all()
    ref = np.linalg.inv(At.double().cpu().numpy())
    err = np.abs(X.double().cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err < 2e-5, err
    # the SIMT kernels on the same input agree to FP32 rounding
    policy.hps_inverse_policy(0)
    Xs = nat.inverse(At)
    policy.hps_inverse_policy(2)
    assert np.abs(Xs.double().cpu().numpy() - X.double().cpu().numpy()).max() / np.abs(ref).max() < 4e-5


def test_tc_inverse_strided_and_batched_over_sms(cuda, policy):
    n, batch = 150, 400
    rng = np.random.default_rng(3)
    A = _mats(rng, batch, n)
    big = torch.zeros((batch, n + 3, n + 5), dtype=torch.float32, device=cuda)
    big[:, :n, :n] = torch.as_tensor(A, dtype=torch.float32)
    Av = big[:, :n, :n]                                   # lda = n + 5, stride = (n+3)(n+5)
    out = torch.full((batch, n, n + 2), float("nan"), dtype=torch.float32, device=cuda)
    Xv = out[:, :, :n]
    nat.inverse(Av, out=Xv)
    torch.cuda.synchronize()
    assert torch.isnan(out[:, :, n:]).all()                 # nothing written past the rows
    ref = np.linalg.inv(A)
    err = np.abs(Xv.double().cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err < 2e-5, err


def test_tc_inverse_singular_sets_info(cuda, policy):
    n = 140
    rng = np.random.default_rng(8)
    A = _mats(rng, 3, n)
    A[1, :, 57] = 0.0          # matrix 1: column 57 is zero
    At = torch.as_tensor(A, dtype=torch.float32, device=cuda)
    info = torch.zeros(3, dtype=torch.int32, device=cuda)
    X = nat.inverse(At, info=info)
    torch.cuda.synchronize()
    inf = info.cpu().numpy()
    assert inf[0] == 0 and inf[2] == 0 and inf[1] == 58
    ref = np.linalg.inv(A[[0, 2]])
    got = X.double().cpu().numpy()[[0, 2]]
    assert np.abs(got - ref).max() / np.abs(ref).max() < 2e-5
    assert np.isfinite(X.cpu().numpy()[1]).all()          # zero pivots are skipped, no inf / nan


def test_inverse_policy_switch(cuda):
    lib = nat.load_library()
    old = lib.hps_inverse_policy(0)
    assert lib.hps_inverse_policy(1) == 0
    assert lib.hps_inverse_policy(2) == 1
    assert lib.hps_inverse_policy(5) == -1
    lib.hps_inverse_policy(old)


def test_tc_inverse_of_leaf_operators(cuda, policy):
    """The interior blocks A_ii of 2D leaf operators at a small leaf size
    (p = 16, half side 2/256): entries up to ~7e7 against an inverse of
    ~1e-6, where an update that cancels the tableau against itself in the
    tensor core would lose every digit."""
    from oracle import hps_oracle as O

    p, half = 16, 2.0 / 256
    _, _, dxx, dyy, _ = O.diff_operators_2D(p, half)
    ncb = 4 * (p - 1)
    rng = np.random.default_rng(4)
    A = np.stack([(dxx + dyy + np.diag(1 + rng.random(p * p)))[ncb:, ncb:] for _ in range(200)])
    At = torch.as_tensor(A, dtype=torch.float32, device=cuda)
    X = nat.inverse(At).double().cpu().numpy()
    ref = np.linalg.inv(At.double().cpu().numpy())
    err = (np.abs(X - ref).max(axis=(1, 2)) / np.abs(ref).max(axis=(1, 2))).max()
    assert err < 2e-5, err


def test_default_policy_uses_the_kernel_for_leaves_only(cuda):
    """At the default policy a plain hps_inverse_batched call (the merges'
    path) stays on the SIMT kernels while the leaf stage's inverse takes the
    tensor-memory kernel; the two leaf inverses agree to FP32 rounding."""
    import jaxhps_gb300 as hps
    from jaxhps_gb300 import _stages as st

    lib = nat.load_library()
    old = lib.hps_inverse_policy(1)
    try:
        dom = hps.Domain(p=16, q=14, root=hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0), L=2)
        x = dom.interior_points
        ones = np.ones(x.shape[:2])
        pde = hps.PDEProblem(dom, source=np.sin(x[..., 0]), D_xx_coefficients=ones, D_yy_coefficients=ones,
                             I_coefficients=1.0 + x[..., 1] ** 2)
        *_, A_tc = st._local_solve_dtn(pde, pde.P, pde.Q, cuda, torch.float32, True, want_source=False)
        lib.hps_inverse_policy(0)
        *_, A_simt = st._local_solve_dtn(pde, pde.P, pde.Q, cuda, torch.float32, True, want_source=False)
        d = (A_tc.double() - A_simt.double()).abs().max() / A_simt.double().abs().max()
        assert float(d) < 2e-5
    finally:
        lib.hps_inverse_policy(old)

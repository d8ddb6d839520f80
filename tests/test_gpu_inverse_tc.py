"""The FP32 batched inverse whose Gauss-Jordan tableau lives in tensor memory
(tcgen05 3xTF32 trailing updates), through the C ABI (hps_inverse_batched):
against numpy.linalg.inv in FP64 and against the SIMT kernels
(hps_inverse_policy(0)), on sizes across one and two 128-row halves, strided
inputs, a singular matrix, and the policy switch.

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
    lib = nat.load_library()
    old = lib.hps_inverse_policy(1)
    yield lib
    lib.hps_inverse_policy(old)


@pytest.mark.parametrize("n,batch", [(65, 3), (100, 7), (128, 5), (129, 4), (196, 300), (200, 2), (256, 3)])
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
    policy.hps_inverse_policy(1)
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
    assert lib.hps_inverse_policy(5) == -1
    lib.hps_inverse_policy(old)

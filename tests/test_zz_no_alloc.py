"""GPU test of hps_inverse_batched_static, the inverse entry point that
allocates nothing (its scratch is a fixed static device array).

Checked through the C ABI against hps_inverse_batched with a caller
workspace, on two calls in a row with different inputs (the second call
runs on scratch that still holds the first call's contents): both run the
same kernels in the same order, so the results must be bitwise equal.  Each
result is also compared with numpy.linalg.inv.  A larger call followed by a
smaller one leaves stale data past the smaller call's scratch layout, which
must not reach its result.  Plus the size-limit rejection.  This file is
named to be collected last.
"""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

# same tolerances as the inverse tests: relative to the result's max entry
CASES = [
    ("f64", torch.float64, 0, 1e-12, 300, 3),   # blocked path (uses scratch)
    ("f32", torch.float32, 1, 2e-5, 420, 2),    # blocked path (uses scratch)
    ("c128", torch.complex128, 2, 1e-12, 90, 2),  # blocked path for c128 (> 64)
    ("f64", torch.float64, 0, 1e-12, 100, 4),   # shared-memory path (no scratch)
]


def _bind():
    from jaxhps_gb300 import _native as nat

    lib = nat.load_library()
    f = lib.hps_inverse_batched_static
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_longlong, C.c_void_p, C.c_longlong,
                  C.c_longlong, C.c_int, C.c_void_p, C.c_void_p]
    return nat, f


def _matrices(rng, batch, n, tdt):
    A = rng.standard_normal((batch, n, n)) + 2 * np.sqrt(n) * np.eye(n)
    if tdt.is_complex:
        A = A + 1j * rng.standard_normal((batch, n, n))
    A = np.ascontiguousarray(A[:, rng.permutation(n), :])
    return torch.as_tensor(A).to(tdt).contiguous()


@pytest.mark.parametrize("name,tdt,code,tol,n,batch", CASES)
def test_static_inverse_matches_workspace_inverse(cuda, name, tdt, code, tol, n, batch):
    nat, f = _bind()
    rng = np.random.default_rng(1000 + n)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    for call in range(2):
        A = _matrices(rng, batch, n, tdt).to(cuda)
        X_ref = torch.empty_like(A)
        info_ref = torch.full((batch,), -7, dtype=torch.int32, device=cuda)
        nat.inverse(A, out=X_ref, info=info_ref)
        X = torch.full_like(A, float("nan"))
        info = torch.full((batch,), -7, dtype=torch.int32, device=cuda)
        st = f(code, n, A.data_ptr(), A.stride(1), A.stride(0), X.data_ptr(), X.stride(1), X.stride(0), batch,
               info.data_ptr(), stream)
        nat.check(st, "hps_inverse_batched_static")
        torch.cuda.synchronize(cuda)
        assert (info.cpu().numpy() == 0).all() and (info_ref.cpu().numpy() == 0).all()
        assert torch.equal(X, X_ref), call
        a = X.cpu().numpy()
        assert np.isfinite(a).all()
        ref = np.linalg.inv(A.cpu().numpy().astype(np.complex128 if tdt.is_complex else np.float64))
        rel = np.abs(a - ref).max() / np.abs(ref).max()
        assert rel < tol, (call, rel)


def test_static_inverse_after_a_larger_call(cuda):
    """A big call fills more of the shared scratch than the small call that
    follows it reads; the small call's result must not depend on that."""
    nat, f = _bind()
    stream = torch.cuda.current_stream(cuda).cuda_stream
    results = []
    for n, batch in ((600, 3), (260, 2), (600, 3), (260, 2)):
        A = _matrices(np.random.default_rng(n), batch, n, torch.float64).to(cuda)
        X = torch.full_like(A, float("nan"))
        info = torch.full((batch,), -7, dtype=torch.int32, device=cuda)
        st = f(0, n, A.data_ptr(), A.stride(1), A.stride(0), X.data_ptr(), X.stride(1), X.stride(0), batch,
               info.data_ptr(), stream)
        nat.check(st, "hps_inverse_batched_static")
        torch.cuda.synchronize(cuda)
        assert (info.cpu().numpy() == 0).all()
        results.append(X.clone())
    assert torch.equal(results[0], results[2]) and torch.equal(results[1], results[3])


def test_static_inverse_rejects_oversize(cuda):
    nat, f = _bind()
    lib = nat.load_library()
    n, batch = 4000, 1   # FP64 blocked workspace ~ 8 n^2 bytes = 128 MB > 64 MiB
    need = lib.hps_inverse_workspace_size(0, n, batch)
    assert need > (64 << 20)
    A = torch.zeros(4, dtype=torch.float64, device=cuda)   # never touched: rejected before any launch
    st = f(0, n, A.data_ptr(), n, n * n, A.data_ptr(), n, n * n, batch, None, None)
    assert st == 4   # HPS_ERR_WORKSPACE
    buf = C.create_string_buffer(512)
    lib.hps_last_error(buf, 512)
    assert b"static scratch" in buf.value

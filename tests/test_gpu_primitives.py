"""GPU tests of the batched primitives behind the C ABI: GEMM and the
Gauss-Jordan inverse (register-resident and blocked paths), every dtype."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DT = {
    "f64": (torch.float64, np.float64, 1e-12),
    "f32": (torch.float32, np.float32, 2e-5),
    "c128": (torch.complex128, np.complex128, 1e-12),
    "c64": (torch.complex64, np.complex64, 2e-5),
}


def _rand(rng, shape, npdt):
    a = rng.standard_normal(shape)
    if np.issubdtype(npdt, np.complexfloating):
        a = a + 1j * rng.standard_normal(shape)
    return a.astype(npdt)


@pytest.mark.parametrize("dt", list(DT))
@pytest.mark.parametrize("m,n,k,batch", [(1, 1, 1, 1), (56, 56, 256, 7), (130, 129, 67, 3), (300, 200, 5, 2),
                                         (5, 9, 0, 2)])
def test_gemm_batched(cuda, dt, m, n, k, batch):
    from jaxhps_gb300 import _native as nat

    tdt, npdt, tol = DT[dt]
    rng = np.random.default_rng(m * 7 + n)
    A = _rand(rng, (batch, m, k), npdt)
    B = _rand(rng, (batch, k, n), npdt)
    Cm = _rand(rng, (batch, m, n), npdt)
    tA, tB, tC = (torch.as_tensor(x, device=cuda) for x in (A, B, Cm))
    out = torch.empty((batch, m, n), dtype=tdt, device=cuda)
    nat.gemm(tA, tB, out, alpha=-0.5, beta=2.0, Cmat=tC)
    ref = -0.5 * A.astype(np.complex128) @ B + 2.0 * Cm
    scale = max(1.0, np.abs(ref).max()) * max(1, k) ** 0.5
    assert np.abs(out.cpu().numpy() - ref).max() <= tol * scale * 10
    # broadcast A (stride 0) and in-place C == D
    nat.gemm(tA[0], tB, tC, alpha=1.0, beta=1.0, Cmat=tC)
    ref2 = A[0] @ B + Cm
    assert np.abs(tC.cpu().numpy() - ref2).max() <= tol * scale * 10


@pytest.mark.parametrize("dt", list(DT))
@pytest.mark.parametrize("n,batch", [(1, 3), (5, 4), (36, 9), (64, 2), (65, 2), (100, 3), (129, 2), (160, 2),
                                     (161, 2), (196, 3), (233, 2)])
def test_inverse_batched(cuda, dt, n, batch):
    from jaxhps_gb300 import _native as nat

    tdt, npdt, tol = DT[dt]
    rng = np.random.default_rng(n)
    A = _rand(rng, (batch, n, n), npdt) + (2 * np.sqrt(n)) * np.eye(n, dtype=npdt)
    # permute rows so that pivoting is exercised
    A = A[:, rng.permutation(n), :]
    tA = torch.as_tensor(A, device=cuda)
    info = torch.zeros(batch, dtype=torch.int32, device=cuda)
    X = nat.inverse(tA, info=info).cpu().numpy()
    assert (info.cpu().numpy() == 0).all()
    Xe = np.linalg.inv(A.astype(np.complex128))
    rel = np.abs(X - Xe).max() / np.abs(Xe).max()
    assert rel < tol * 20, rel
    # in place
    nat.inverse(tA, out=tA)
    assert np.allclose(tA.cpu().numpy(), X, atol=tol * 10, rtol=tol * 10)


@pytest.mark.parametrize("n", [40, 300])
def test_inverse_reports_singular(cuda, n):
    from jaxhps_gb300 import _native as nat

    A = np.zeros((2, n, n))
    A[0] = np.eye(n)
    A[1] = np.eye(n)
    A[1, :, 3] = 0.0  # singular: zero column
    tA = torch.as_tensor(A, device=cuda)
    info = torch.zeros(2, dtype=torch.int32, device=cuda)
    nat.inverse(tA, info=info)
    inf = info.cpu().numpy()
    assert inf[0] == 0 and inf[1] > 0


def test_inverse_large_blocked(cuda):
    from jaxhps_gb300 import _native as nat

    n = 1100
    rng = np.random.default_rng(3)
    A = rng.standard_normal((1, n, n)) + np.sqrt(n) * np.eye(n)
    X = nat.inverse(torch.as_tensor(A, device=cuda)).cpu().numpy()
    assert np.abs(X[0] @ A[0] - np.eye(n)).max() < 1e-10


@pytest.mark.parametrize("n,dt", [(3000, "f32"), (2500, "f64"), (700, "c64")])
def test_inverse_large_single_matrix_multi_cta_panel(cuda, n, dt):
    """One large matrix: the panel is split over many CTAs (cooperative launch)."""
    from jaxhps_gb300 import _native as nat

    tdt, npdt, tol = DT[dt]
    rng = np.random.default_rng(n)
    A = _rand(rng, (1, n, n), npdt) + (2 * np.sqrt(n)) * np.eye(n, dtype=npdt)
    A = np.ascontiguousarray(A[:, rng.permutation(n), :])
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    X = nat.inverse(torch.as_tensor(A, device=cuda), info=info).cpu().numpy()
    assert int(info.item()) == 0
    Xe = np.linalg.inv(A.astype(np.complex128 if np.iscomplexobj(A) else np.float64))
    rel = np.abs(X - Xe).max() / np.abs(Xe).max()
    assert rel < tol * 20, rel


@pytest.mark.parametrize("m,n,k,batch,odd", [(196, 64, 196, 3, False), (300, 200, 150, 2, False), (257, 33, 131, 2, True),
                                             (1100, 300, 257, 1, False)])
def test_gemm_tensor_core_path(cuda, m, n, k, batch, odd):
    """FP32 products on the tcgen05 kernel (3xTF32; forced with
    hps_gemm_policy(2)): FP32-level accuracy, ragged tiles, unaligned leading
    dimensions, C aliasing D."""
    from jaxhps_gb300 import _native as nat

    L = nat.load_library()
    old_policy = L.hps_gemm_policy(2)

    rng = np.random.default_rng(m + n + k)
    pad = 1 if odd else 0
    Ab = rng.standard_normal((batch, m, k + pad)).astype(np.float32)
    B = rng.standard_normal((batch, k, n)).astype(np.float32)
    Cm = rng.standard_normal((batch, m, n)).astype(np.float32)
    tA = torch.as_tensor(Ab, device=cuda)[:, :, :k]          # lda = k + 1 when odd: unaligned rows
    tB, tC = torch.as_tensor(B, device=cuda), torch.as_tensor(Cm, device=cuda)
    try:
        nat.gemm(tA, tB, tC, alpha=0.75, beta=-1.25, Cmat=tC)    # in place
        torch.cuda.synchronize()
    finally:
        L.hps_gemm_policy(old_policy)
    ref = 0.75 * (Ab[:, :, :k].astype(np.float64) @ B) - 1.25 * Cm
    err = np.abs(tC.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err < 2e-6 * max(1.0, np.sqrt(k / 64)), err
    assert nat.load_library().hps_gemm_tc_status() == 0


@pytest.mark.parametrize("m,n,k,batch,odd", [(196, 64, 196, 3, False), (300, 20, 150, 2, False), (257, 33, 131, 2, True),
                                             (1100, 300, 257, 1, False)])
def test_gemm_tensor_core_complex64(cuda, m, n, k, batch, odd):
    """complex64 products on the tcgen05 kernel (one real product of the
    interleaved A with the 2x2-block expansion of B; forced with
    hps_gemm_policy(2)): complex64-level accuracy, ragged tiles, unaligned
    leading dimensions, C aliasing D."""
    from jaxhps_gb300 import _native as nat

    L = nat.load_library()
    old_policy = L.hps_gemm_policy(2)

    rng = np.random.default_rng(m + n + k + 1)
    pad = 1 if odd else 0

    def cr(*shape):
        return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)

    Ab, B, Cm = cr(batch, m, k + pad), cr(batch, k, n), cr(batch, m, n)
    tA = torch.as_tensor(Ab, device=cuda)[:, :, :k]
    tB, tC = torch.as_tensor(B, device=cuda), torch.as_tensor(Cm, device=cuda)
    try:
        nat.gemm(tA, tB, tC, alpha=0.75, beta=-1.25, Cmat=tC)
        torch.cuda.synchronize()
    finally:
        L.hps_gemm_policy(old_policy)
    ref = 0.75 * (Ab[:, :, :k].astype(np.complex128) @ B) - 1.25 * Cm
    err = np.abs(tC.cpu().numpy() - ref).max() / np.abs(ref).max()
    # FP32 accumulation over the 2k real terms of each complex dot product
    assert err < 2e-6 * max(1.0, np.sqrt(2 * k / 64)), err
    assert nat.load_library().hps_gemm_tc_status() == 0


@pytest.mark.parametrize("dt,m,n,k,batch", [("c64", 56, 14, 14, 3), ("f32", 5, 3, 7, 2), ("f32", 56, 64, 256, 2),
                                            ("c64", 130, 33, 17, 2), ("c64", 256, 56, 60, 4), ("f32", 64, 1, 40, 3)])
def test_gemm_policy_every_product_on_tensor_cores(cuda, dt, m, n, k, batch):
    """hps_gemm_policy(2) sends every FP32 / complex64 product to the tcgen05
    kernel, including tiles far below its 128-row tile and K below one
    K-step: results stay at FP32 accuracy; the policy is restored."""
    from jaxhps_gb300 import _native as nat

    L = nat.load_library()
    rng = np.random.default_rng(m * n + k)
    if dt == "c64":
        def r(*s):
            return (rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64)
    else:
        def r(*s):
            return rng.standard_normal(s).astype(np.float32)
    A, B, Cm = r(batch, m, k), r(batch, k, n), r(batch, m, n)
    tA, tB, tC = (torch.as_tensor(x, device=cuda) for x in (A, B, Cm))
    old = L.hps_gemm_policy(2)
    try:
        nat.gemm(tA, tB, tC, alpha=1.5, beta=0.5, Cmat=tC)
        torch.cuda.synchronize()
    finally:
        L.hps_gemm_policy(old)
    assert old == 1
    ref = 1.5 * (A.astype(np.complex128) @ B) + 0.5 * Cm
    err = np.abs(tC.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err < 3e-6 * max(1.0, np.sqrt(2 * k / 64)), err
    assert L.hps_gemm_tc_status() == 0


@pytest.mark.parametrize("m,n,k,batch,pad", [(196, 64, 196, 160, 0), (196, 56, 60, 200, 0), (56, 64, 256, 400, 0),
                                             (130, 129, 67, 120, 0), (200, 37, 50, 200, 0), (100, 48, 33, 400, 1),
                                             (97, 97, 9, 130, 3)])
def test_gemm_f32_vector_tiles_match_scalar_tiles(cuda, m, n, k, batch, pad):
    """The FP32 8x8 tiles with 16-byte shared loads (default) against the
    same tiles with 4-byte loads (policy 3): the FMA order per output is the
    same, so the results are identical, for tile-aligned and ragged M, N, K,
    leading dimensions that are not multiples of 4 (pad > 0: scalar global
    loads), a broadcast A and C == D in place.  Both against NumPy too."""
    from jaxhps_gb300 import _native as nat

    L = nat.load_library()
    rng = np.random.default_rng(m + 3 * n + 7 * k)
    A = rng.standard_normal((batch, m, k + pad)).astype(np.float32)
    B = rng.standard_normal((batch, k, n + pad)).astype(np.float32)
    Cm = rng.standard_normal((batch, m, n + pad)).astype(np.float32)
    tA = torch.as_tensor(A, device=cuda)[:, :, :k]
    tB = torch.as_tensor(B, device=cuda)[:, :, :n]
    outs = []
    for pol in (0, 3):
        old = L.hps_gemm_policy(pol)
        try:
            tC = torch.as_tensor(Cm, device=cuda)[:, :, :n]
            out = torch.empty((batch, m, n + pad), dtype=torch.float32, device=cuda)[:, :, :n]
            nat.gemm(tA, tB, out, alpha=-0.75, beta=1.5, Cmat=tC)
            nat.gemm(tA[0], tB, tC, alpha=1.0, beta=1.0, Cmat=tC)     # broadcast A, in place
            torch.cuda.synchronize()
        finally:
            L.hps_gemm_policy(old)
        outs.append((out.cpu().numpy(), tC.cpu().numpy()))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
    A64, B64, C64 = A[:, :, :k].astype(np.float64), B[:, :, :n].astype(np.float64), Cm[:, :, :n].astype(np.float64)
    ref = -0.75 * A64 @ B64 + 1.5 * C64
    ref2 = A64[0] @ B64 + C64
    scale = max(1.0, np.abs(ref).max()) * max(1, k) ** 0.5
    assert np.abs(outs[0][0] - ref).max() <= 2e-5 * scale * 10
    assert np.abs(outs[0][1] - ref2).max() <= 2e-5 * scale * 10


@pytest.mark.parametrize("m,n,k,batch,pad", [(3584, 64, 3584, 1, 0), (1792, 64, 1792, 4, 0), (896, 64, 896, 16, 0),
                                             (100, 37, 2000, 3, 0), (64, 14, 600, 2, 0), (130, 96, 1031, 2, 1),
                                             (70, 64, 515, 5, 3)])
def test_gemm_f32_cluster_split_k(cuda, m, n, k, batch, pad):
    """FP32 products with few output tiles and a long K run split-K over the
    CTAs of a thread-block cluster (partial tiles reduced in rank order
    through distributed shared memory): FP32 accuracy against NumPy, the
    same bits on every run, ragged M / N / K, leading dimensions that are not
    multiples of 4, a broadcast A and C == D in place."""
    from jaxhps_gb300 import _native as nat

    rng = np.random.default_rng(m + n + k)
    A = rng.standard_normal((batch, m, k + pad)).astype(np.float32)
    B = rng.standard_normal((batch, k, n + pad)).astype(np.float32)
    Cm = rng.standard_normal((batch, m, n + pad)).astype(np.float32)
    tA = torch.as_tensor(A, device=cuda)[:, :, :k]
    tB = torch.as_tensor(B, device=cuda)[:, :, :n]
    runs = []
    for _ in range(2):
        tC = torch.as_tensor(Cm, device=cuda)[:, :, :n]
        out = torch.empty((batch, m, n + pad), dtype=torch.float32, device=cuda)[:, :, :n]
        nat.gemm(tA, tB, out, alpha=0.5, beta=-1.0, Cmat=tC)
        nat.gemm(tA[0], tB, tC, alpha=1.0, beta=1.0, Cmat=tC)
        torch.cuda.synchronize()
        runs.append((out.cpu().numpy(), tC.cpu().numpy()))
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])
    A64, B64, C64 = A[:, :, :k].astype(np.float64), B[:, :, :n].astype(np.float64), Cm[:, :, :n].astype(np.float64)
    ref = 0.5 * A64 @ B64 - C64
    ref2 = A64[0] @ B64 + C64
    scale = max(1.0, np.abs(ref).max()) * k ** 0.5
    assert np.abs(runs[0][0] - ref).max() <= 2e-5 * scale * 10
    assert np.abs(runs[0][1] - ref2).max() <= 2e-5 * scale * 10


@pytest.mark.parametrize("M,N,K,batch,bcastA,viewA,inplace", [
    (196, 64, 196, 600, False, False, False),   # the leaf solve v = inv(A_ii) r: two row tiles, K tail
    (196, 56, 56, 300, False, True, True),      # du = Y_int g + v: A a row-offset view, C aliasing D, N tail
    (56, 64, 196, 300, True, False, False),     # h = Q_int v: broadcast A, one partial row tile
    (300, 48, 100, 5, False, False, False),
    (128, 64, 32, 1, False, False, True),
    (200, 16, 12, 7, False, False, False),      # K shorter than one K-tile
])
def test_gemm_tma_warp_specialised(cuda, M, N, K, batch, bcastA, viewA, inplace):
    """Variant 8 (TMA loads, warp-specialised tcgen05 3xTF32) against an FP64
    product, FP32-level tolerance (1e-5 relative), with the operand layouts
    the leaf products use; no bounded wait may run out."""
    from jaxhps_gb300 import _native as nat

    lib = nat.lib()
    g = torch.Generator(device=cuda).manual_seed(M * 7 + N)
    if bcastA:
        A = torch.randn(M, K, device=cuda, generator=g)
        A64 = A.double().expand(batch, M, K)
    elif viewA:
        big = torch.randn(batch, M + 60, K, device=cuda, generator=g)
        A = big[:, 60:, :]
        A64 = A.double()
    else:
        A = torch.randn(batch, M, K, device=cuda, generator=g)
        A64 = A.double()
    B = torch.randn(batch, K, N, device=cuda, generator=g)
    Cm = torch.randn(batch, M, N, device=cuda, generator=g)
    ref = (A64 @ B.double()) * 0.75 + Cm.double() * 1.5
    lib.hps_gemm_tc_status_reset()
    old = lib.hps_gemm_force_variant(8)
    try:
        D = Cm.clone() if inplace else torch.full((batch, M, N), float("nan"), device=cuda)
        nat.gemm(A, B, D, alpha=0.75, beta=1.5, Cmat=D if inplace else Cm, batch=batch)
        torch.cuda.synchronize()
    finally:
        lib.hps_gemm_force_variant(old)
    err = float((D.double() - ref).abs().max() / ref.abs().max())
    assert err < 1e-5, err
    assert lib.hps_gemm_tc_status() == 0

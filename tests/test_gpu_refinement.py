"""GPU tests of mixed precision: the FP64 residual kernel against dense
NumPy, and FP32-build + FP64-residual refinement against the FP64 oracle.

Tolerance for the refined solution: relative max error <= 1e-10 against the
FP64 oracle (the target stated for the mixed path)."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300 import _refinement as rf
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


def _setup(L, p, q, nsrc, extra, seed=0):
    rng = np.random.default_rng(seed)
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=root, L=L)
    x = dom.interior_points
    c = 1.0 + 0.5 * np.exp(-((x[..., 0] - 0.2) ** 2 + (x[..., 1] + 0.3) ** 2) / 0.04)
    ones = np.ones_like(c)
    coeffs = {"D_xx": ones, "D_yy": ones, "I": c}
    kw = dict(D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c)
    if extra:
        bx = 0.3 * np.sin(x[..., 1])
        bxy = 0.2 * np.cos(x[..., 0])
        coeffs.update({"D_x": bx, "D_xy": bxy})
        kw.update(D_x_coefficients=bx, D_xy_coefficients=bxy)
    shape = x.shape[:2] + ((nsrc,) if nsrc else ())
    f = rng.standard_normal(shape)
    return dom, hps.PDEProblem(dom, source=f, **kw), O.Problem2D(root.bounds, L, p, q, coeffs, f)


@pytest.mark.parametrize("extra", [False, True])
def test_residual_kernel_matches_dense(cuda, extra):
    L, p, q, ns = 2, 8, 6, 3
    dom, pde, ref = _setup(L, p, q, ns, extra)
    hps.build_solver(pde, precision="mixed")
    state = pde._state
    rng = np.random.default_rng(1)
    nl, ncb = dom.n_leaves, 4 * (p - 1)
    u_int = rng.standard_normal((nl, p * p - ncb, ns))
    g = rng.standard_normal((nl, 4 * q, ns))
    tu = torch.as_tensor(u_int, device=cuda)
    tg = torch.as_tensor(g, device=cuda)
    r32 = torch.empty(u_int.shape, dtype=torch.float32, device=cuda)
    flux = torch.empty(g.shape, dtype=torch.float64, device=cuda)
    ufull = torch.empty((nl, p * p, ns), dtype=torch.float64, device=cuda)
    rf._residual(state, tu, tg, r32, flux, u_full=ufull)
    A = O.assemble_operator(ref.coeffs, ref.ops, nl, p * p)
    full = np.concatenate([np.einsum("ij,ljs->lis", ref.P, g), u_int], axis=1)
    r_ref = ref.source[:, ncb:] - np.einsum("lij,ljs->lis", A[:, ncb:, :], full)
    F_ref = np.einsum("ij,ljs->lis", ref.Q, full)
    assert np.allclose(ufull.cpu().numpy(), full, atol=1e-12)
    scale = np.abs(r_ref).max()
    assert np.abs(r32.cpu().numpy() - r_ref).max() < 1e-6 * scale
    assert np.abs(flux.cpu().numpy() - F_ref).max() < 1e-11 * np.abs(F_ref).max()


@pytest.mark.parametrize("L,p,q,nsrc,extra", [(2, 8, 6, None, False), (3, 12, 10, 4, True), (3, 16, 14, 2, False)])
def test_mixed_matches_fp64_oracle(cuda, L, p, q, nsrc, extra):
    dom, pde, ref = _setup(L, p, q, nsrc, extra, seed=2)
    hps.build_solver(pde, precision="mixed")
    bp = dom.boundary_points
    g = np.sin(bp[:, 0]) + bp[:, 1] ** 2
    if nsrc:
        g = np.stack([g * (k + 1) for k in range(nsrc)], -1)
    u = hps.solve(pde, g).numpy()
    ur = ref.build().solve(g)
    assert u.shape == ur.shape
    err = np.abs(u - ur).max() / np.abs(ur).max()
    hist = pde._state.history
    assert err < 1e-10, (err, hist)
    assert len(hist) < pde._state.max_iters


@pytest.mark.parametrize("extra", [False, True])
def test_incremental_residual_matches_fp64(cuda, extra):
    """r(x) - J dx evaluated in double-float equals the FP64 residual r(x + dx)."""
    L, p, q, ns = 2, 10, 8, 5
    dom, pde, ref = _setup(L, p, q, ns, extra, seed=3)
    hps.build_solver(pde, precision="mixed")
    state = pde._state
    rng = np.random.default_rng(4)
    nl, ncb = dom.n_leaves, 4 * (p - 1)
    ni = p * p - ncb
    u = torch.as_tensor(rng.standard_normal((nl, ni, ns)), device=cuda)
    g = torch.as_tensor(rng.standard_normal((nl, 4 * q, ns)), device=cuda)
    du = torch.as_tensor(1e-2 * rng.standard_normal((nl, ni, ns)), device=cuda, dtype=torch.float32)
    dg = torch.as_tensor(1e-2 * rng.standard_normal((nl, 4 * q, ns)), device=cuda, dtype=torch.float32)
    r32 = torch.empty((nl, ni, ns), dtype=torch.float32, device=cuda)
    r64 = torch.empty((nl, ni, ns), dtype=torch.float64, device=cuda)
    flux = torch.empty((nl, 4 * q, ns), dtype=torch.float64, device=cuda)
    rf._residual(state, u, g, r32, flux, r64=r64)
    rf._residual_update(state, du, dg, r64, r32, flux)
    r64b = torch.empty_like(r64)
    flux_b = torch.empty_like(flux)
    rf._residual(state, u + du.double(), g + dg.double(), r32, flux_b, r64=r64b)
    # the update's rounding is relative to the size of A du, not of r
    ref_d = torch.empty_like(r64)
    fl_d = torch.empty_like(flux)
    rf._residual(state, du.double(), dg.double(), r32, fl_d, r64=ref_d, zero_source=True)
    scale_r = float(ref_d.abs().max())
    scale_f = float(fl_d.abs().max())
    assert float((r64 - r64b).abs().max()) < 1e-10 * scale_r
    assert float((flux - flux_b).abs().max()) < 1e-10 * scale_f


@pytest.mark.parametrize("p,ns,extra", [(10, 5, False), (16, 20, False), (12, 3, True), (16, 64, True)])
def test_pair_residual_update_matches_fp64(cuda, p, ns, extra):
    """The FP32-pair residual: its FP64 start equals hps_residual_2d split in
    two, and after r -= J dx (one grid line per thread) it equals the FP64
    residual at x + dx, within the update's rounding relative to |J dx|; the
    update agrees with the FP64-storage update kernel."""
    L, q = 2, p - 2
    assert hps._native.lib().hps_residual_df_supported(p, q) == 1
    dom, pde, ref = _setup(L, p, q, ns, extra, seed=7)
    hps.build_solver(pde, precision="mixed")
    state = pde._state
    rng = np.random.default_rng(8)
    nl, ncb = dom.n_leaves, 4 * (p - 1)
    ni = p * p - ncb
    u = torch.as_tensor(rng.standard_normal((nl, ni, ns)), device=cuda)
    g = torch.as_tensor(rng.standard_normal((nl, 4 * q, ns)), device=cuda)
    du = torch.as_tensor(1e-2 * rng.standard_normal((nl, ni, ns)), device=cuda, dtype=torch.float32)
    dg = torch.as_tensor(1e-2 * rng.standard_normal((nl, 4 * q, ns)), device=cuda, dtype=torch.float32)
    r32 = torch.empty((nl, ni, ns), dtype=torch.float32, device=cuda)
    r_lo = torch.empty_like(r32)
    r64 = torch.empty((nl, ni, ns), dtype=torch.float64, device=cuda)
    flux = torch.empty((nl, 4 * q, ns), dtype=torch.float64, device=cuda)
    rf._residual(state, u, g, r32, flux, r64=r64, r_lo=r_lo)
    pair = r32.double() + r_lo.double()
    assert float((pair - r64).abs().max()) <= 2.0 ** -46 * float(r64.abs().max())
    flux_old = flux.clone()
    r32_old = torch.empty_like(r32)
    rf._residual_update(state, du, dg, r64, r32_old, flux_old)
    prep = rf._df_prepare(rf._res_args(state, None, None, r32, flux))
    rf._residual_update_df(state, prep, du, dg, r_lo, r32, flux)
    r64b = torch.empty_like(r64)
    flux_b = torch.empty_like(flux)
    rf._residual(state, u + du.double(), g + dg.double(), r32_old, flux_b, r64=r64b)
    ref_d = torch.empty_like(r64)
    fl_d = torch.empty_like(flux)
    rf._residual(state, du.double(), dg.double(), r32_old, fl_d, r64=ref_d, zero_source=True)
    scale_r = float(ref_d.abs().max())
    scale_f = float(fl_d.abs().max())
    pair = r32.double() + r_lo.double()
    assert float((pair - r64b).abs().max()) < 1e-10 * scale_r
    assert float((pair - r64).abs().max()) < 1e-12 * scale_r
    assert float((flux - flux_b).abs().max()) < 1e-10 * scale_f
    assert float((flux - flux_old).abs().max()) < 1e-12 * scale_f


def test_pinned_source_upload_matches_numpy_source(cuda):
    """A page-locked CPU source is copied on a side stream while the build
    runs; the solution is bit-identical to the one from a NumPy source."""
    L, p, q, ns = 3, 12, 10, 4
    dom, pde, _ = _setup(L, p, q, ns, True, seed=5)
    bp = dom.boundary_points
    g = np.stack([np.cos(bp[:, 0]) * (k + 1) for k in range(ns)], -1)
    hps.build_solver(pde, precision="mixed")
    u_np = hps.solve(pde, g).numpy()
    f_pin = torch.as_tensor(pde.source).pin_memory()
    dom2, pde2, _ = _setup(L, p, q, ns, True, seed=5)
    pde2.source = f_pin
    hps.build_solver(pde2, precision="mixed")
    u_pin = hps.solve(pde2, g).numpy()
    assert np.array_equal(u_np, u_pin)
    assert len(pde2._state.history) == len(pde._state.history)
    # the result read into a page-locked buffer the caller keeps
    buf = torch.empty(u_np.shape, dtype=torch.float64).pin_memory()
    hps.build_solver(pde2, precision="mixed")
    r = hps.solve(pde2, g, out=buf)
    assert r is buf and np.array_equal(buf.numpy(), u_np)


def test_solution_assembled_into_caller_buffers(cuda):
    """One right-hand side: a page-locked `out` is written by the assembly
    kernel through its device mapping, a pageable one by a copy; both equal
    the solution returned on the host, bit for bit."""
    L, p, q = 3, 12, 10
    dom, pde, _ = _setup(L, p, q, None, False, seed=9)
    bp = dom.boundary_points
    g = np.cos(bp[:, 0]) - bp[:, 1]
    hps.build_solver(pde, precision="mixed")
    u_ref = hps.solve(pde, g).numpy()
    pinned = torch.full(u_ref.shape, float("nan"), dtype=torch.float64).pin_memory()
    pageable = torch.full(u_ref.shape, float("nan"), dtype=torch.float64)
    assert hps.solve(pde, g, out=pinned) is pinned
    assert hps.solve(pde, g, out=pageable) is pageable
    assert np.array_equal(pinned.numpy(), u_ref)
    assert np.array_equal(pageable.numpy(), u_ref)


def test_pair_accumulator_matches_fp64(cuda):
    """(hi, lo) += dx over several corrections of shrinking size equals the
    FP64 sum to double-float rounding; the maxima are max |dx| and max |x|."""
    from jaxhps_gb300 import _native as nat

    rng = np.random.default_rng(12)
    n = 4 * 12345
    hi = torch.zeros(n, dtype=torch.float32, device=cuda)
    lo = torch.zeros_like(hi)
    ref = np.zeros(n)
    out = torch.empty(2, dtype=torch.float64, device=cuda)
    for k in range(5):
        dx = (rng.standard_normal(n) * 10.0 ** (-3 * k)).astype(np.float32)
        mx, my = nat.accumulate_max_df(torch.as_tensor(dx, device=cuda), hi, lo, out)
        ref += dx.astype(np.float64)
        assert mx == float(np.abs(dx).max())
        assert abs(my - np.abs(ref).max()) <= 1e-6 * np.abs(ref).max()
    got = hi.double().cpu().numpy() + lo.double().cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()


def _boundary_interp_ref(Pside, g, p, q):
    """FP64 Chebyshev-boundary values of every leaf from its Gauss boundary
    data: point k of the exterior-first order lies on one side (two at the
    corners, averaged), side s holding points s(p-1) .. s(p-1)+p-1 (mod ncb)."""
    ncb = 4 * (p - 1)
    out = np.zeros((g.shape[0], ncb, g.shape[2]))
    cnt = np.zeros(ncb)
    for side in range(4):
        for t in range(p):
            k = (side * (p - 1) + t) % ncb
            out[:, k] += np.einsum("j,ljs->ls", Pside[t], g[:, side * q:(side + 1) * q])
            cnt[k] += 1
    return out / cnt[None, :, None]


@pytest.mark.parametrize("p,q,ns", [(16, 14, 64), (12, 10, 3), (7, 5, 40)])
def test_pair_assembly_matches_fp64(cuda, p, q, ns):
    """hps_assemble_u_2d_df: the interior is hi + lo exactly, the boundary the
    FP64 interpolation of g to double-float accuracy (<= 1e-13 relative)."""
    from jaxhps_gb300 import _native as nat

    rng = np.random.default_rng(p * 100 + ns)
    nl, ncb = 37, 4 * (p - 1)
    ni = p * p - ncb
    Pside = rng.standard_normal((p, q))
    hi = rng.standard_normal((nl, ni, ns)).astype(np.float32)
    lo = (rng.standard_normal((nl, ni, ns)) * 1e-8).astype(np.float32)
    g = rng.standard_normal((nl, 4 * q, ns))
    out = torch.full((nl, p * p, ns), float("nan"), dtype=torch.float64, device=cuda)
    t = [torch.as_tensor(a, device=cuda) for a in (Pside, hi, lo, g)]
    nat.check(nat.lib().hps_assemble_u_2d_df(nl, p, q, ns, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(),
                                             t[3].data_ptr(), out.data_ptr(), nat.stream_ptr()),
              "hps_assemble_u_2d_df")
    u = out.cpu().numpy()
    assert np.array_equal(u[:, ncb:], hi.astype(np.float64) + lo.astype(np.float64))
    ref = _boundary_interp_ref(Pside, g, p, q)
    assert np.abs(u[:, :ncb] - ref).max() <= 1e-13 * np.abs(ref).max()

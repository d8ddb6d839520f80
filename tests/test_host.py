"""CPU tests of the host side: operators, grids, index maps, the C ABI's
exported symbols and the API's argument validation.  No GPU work here."""

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import jaxhps_gb300 as hps
from jaxhps_gb300 import _grid_creation_2D as g2
from jaxhps_gb300 import _index_maps as im
from jaxhps_gb300 import _precompute_operators_2D as op2
from jaxhps_gb300 import _quadrature as qd
from oracle import hps_oracle as O

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("p,q", [(6, 4), (8, 6), (16, 14)])
def test_operators_match_oracle(p, q):
    half = 0.37
    mine = op2.precompute_diff_operators_2D(p, half)
    ref = O.diff_operators_2D(p, half)
    for a, b in zip(mine, ref):
        assert np.allclose(a, b, atol=1e-12 * np.abs(b).max())
    assert np.allclose(op2.precompute_P_2D_DtN(p, q), O.P_2D_DtN(p, q), atol=1e-14)
    assert np.allclose(op2.precompute_Q_2D_DtN(p, q, mine[0], mine[1]), O.Q_2D_DtN(p, q, ref[0], ref[1]),
                       rtol=1e-12, atol=1e-10)
    assert np.allclose(op2.precompute_P_2D_ItI(p, q), O.P_2D_ItI(p, q), atol=1e-14)
    N = op2.precompute_N_matrix_2D(mine[0], mine[1], p)
    assert np.allclose(op2.precompute_QH_2D_ItI(N, p, q, 2.5), O.QH_2D_ItI(p, q, ref[0], ref[1], 2.5),
                       rtol=1e-12, atol=1e-10)
    Nt = op2.precompute_N_tilde_matrix_2D(mine[0], mine[1], p)
    assert np.allclose(op2.precompute_G_2D_ItI(Nt, 2.5), O.G_2D_ItI(ref[0], ref[1], p, 2.5), atol=1e-10)


def test_quadrature_matches_oracle():
    for n in (2, 3, 7, 16):
        assert np.allclose(qd.chebyshev_points(n), O.chebyshev_points(n), atol=0)
        x = qd.chebyshev_points(n)
        assert np.allclose(qd.differentiation_matrix_1D(x), O.differentiation_matrix_1D(x), atol=1e-13)
    a, b = qd.gauss_points(7), np.linspace(-1, 1, 11)
    assert np.allclose(qd.barycentric_lagrange_interpolation_matrix_1D(a, b), O.barycentric_matrix_1D(a, b),
                       atol=1e-14)
    c = qd.chebyshev_points(5)
    assert np.allclose(qd.barycentric_lagrange_interpolation_matrix_1D(c, c), np.eye(5))
    w = qd.chebyshev_weights(9, (-1.0, 1.0))
    assert abs(w.sum() - 2.0) < 1e-14
    assert abs(w @ qd.chebyshev_points(9) ** 2 - 2 / 3) < 1e-14


@pytest.mark.parametrize("L,p,q", [(0, 5, 3), (2, 6, 4), (3, 8, 6)])
def test_grids_match_oracle(L, p, q):
    root = hps.DiscretizationNode2D(-1.0, 2.0, 0.5, 3.5)
    dom = hps.Domain(p=p, q=q, root=root, L=L)
    assert np.allclose(dom.interior_points, O.leaf_points_2D(O.uniform_leaf_bounds_2D(root.bounds, L), p))
    assert np.allclose(dom.boundary_points, O.boundary_gauss_points_2D(root.bounds, L, q))
    assert list(g2.rearrange_indices_ext_int(p)) == list(O.ext_first_order_2D(p))
    assert dom.n_leaves == 4 ** L


def _emulate_merge(Ts, hs, maps):
    """NumPy restatement of the merge gather + Schur complement driven by the
    index maps (what hps_merge_level_dtn computes)."""
    Tm, hm = np.stack(Ts), np.stack(hs)
    ni, ne = maps.n_int, maps.n_ext
    D = np.zeros((ni, ni))
    for i in range(ni):
        for t in range(2):
            c, l = maps.int_c[i, t], maps.int_l[i, t]
            for j in range(ni):
                lj = maps.loc[c, j]
                if lj >= 0:
                    D[i, j] += Tm[c, l, lj]
    C = np.zeros((ni, ne))
    B = np.zeros((ne, ni))
    A = np.zeros((ne, ne))
    for x in range(ne):
        c, l = maps.ext_c[x], maps.ext_l[x]
        for i in range(ni):
            li = maps.loc[c, i]
            if li >= 0:
                C[i, x] = Tm[c, li, l]
                B[x, i] = Tm[c, l, li]
        for y in range(ne):
            if maps.ext_c[y] == c:
                A[x, y] = Tm[c, l, maps.ext_l[y]]
    dh = hm[maps.int_c[:, 0], maps.int_l[:, 0]] + hm[maps.int_c[:, 1], maps.int_l[:, 1]]
    hext = hm[maps.ext_c, maps.ext_l]
    Dinv = np.linalg.inv(D)
    S = -Dinv @ C
    gt = -Dinv @ dh
    return S, A + B @ S, hext + B @ gt, gt


@pytest.mark.parametrize("nc", [1, 3, 6])
def test_quad_merge_maps_reproduce_oracle(nc):
    rng = np.random.default_rng(nc)
    n = 4 * nc
    Ts = [rng.standard_normal((n, n)) + 4 * np.eye(n) for _ in range(4)]
    hs = [rng.standard_normal((n, 2)) for _ in range(4)]
    S, T, h, gt = O.quad_merge_dtn(*Ts, *hs)
    maps = im.quad_merge_maps_dtn(nc)
    S2, T2, h2, gt2 = _emulate_merge(Ts, hs, maps)
    assert np.allclose(S, S2) and np.allclose(T, T2) and np.allclose(h, h2) and np.allclose(gt, gt2)


@pytest.mark.parametrize("nc", [1, 4])
def test_down_scatter_maps_reproduce_oracle(nc):
    rng = np.random.default_rng(7)
    S = rng.standard_normal((4 * nc, 8 * nc))
    g = rng.standard_normal((8 * nc, 3))
    gt = rng.standard_normal((4 * nc, 3))
    ref = O._propagate_down_dtn(S, g, gt)
    maps = im.quad_merge_maps_dtn(nc)
    gi = S @ g + gt
    out = np.empty((4, 4 * nc, 3))
    for c in range(4):
        for k in range(4 * nc):
            cd = maps.code[c, k]
            out[c, k] = g[cd] if cd >= 0 else gi[-cd - 1]
    assert np.allclose(out, ref)


def _declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = h.read_text()
        names |= set(re.findall(r"^\s*(?:[\w\*\s]+?)\b(hps_\w+)\s*\(", txt, flags=re.M))
    return names


def test_library_exports_header_symbols():
    from jaxhps_gb300 import _build, _native

    _build.build()
    lib = ctypes.CDLL(str(_native._LIB_PATH))
    declared = _declared_symbols()
    assert len(declared) >= 10
    for name in declared:
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"
    assert set(_native.EXPORTED_SYMBOLS) <= declared
    lib.hps_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.hps_version()


def test_gpu_path_fails_loudly_without_cuda(monkeypatch):
    import torch
    from jaxhps_gb300 import _native

    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    with pytest.raises(_native.NativeError):
        _native.lib()


def test_pdeproblem_validation():
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=6, q=4, root=root, L=1)
    ones = np.ones(dom.interior_points.shape[:2])
    with pytest.raises(ValueError):
        hps.PDEProblem(dom, source=ones, D_xx_coefficients=ones, D_z_coefficients=ones)
    with pytest.raises(ValueError):
        hps.PDEProblem(dom, source=ones, D_xx_coefficients=ones[:2])
    with pytest.raises(ValueError):
        hps.PDEProblem(dom, source=ones, D_xx_coefficients=ones, use_ItI=True)
    pde = hps.PDEProblem(dom, source=ones, D_xx_coefficients=ones, D_yy_coefficients=ones)
    cs, ops = pde.active_coefficients()
    assert len(cs) == 2 and ops[0] is pde.D_xx and ops[1] is pde.D_yy
    assert pde.Y is None and pde.S_lst == []


@pytest.mark.parametrize("L,q", [(1, 4), (3, 6)])
def test_leaf_node_maps(L, q):
    from jaxhps_gb300 import _refinement as rf

    root = hps.DiscretizationNode2D(-1.0, 1.0, -2.0, 0.0)
    dom = hps.Domain(p=q + 2, q=q, root=root, L=L)
    nodes = rf.leaf_gauss_nodes_2D(g2.uniform_leaf_bounds_2D(root.bounds, L), q)
    nbr, bnode = rf.node_maps(nodes, dom.boundary_points, scale=2.0)
    flat = nodes.reshape(-1, 2)
    inner = nbr >= 0
    # symmetric pairing of coinciding nodes
    assert (nbr[nbr[inner]] == np.nonzero(inner)[0]).all()
    assert np.allclose(flat[inner], flat[nbr[inner]])
    # every interior edge node paired, every boundary node mapped once
    assert (~inner).sum() == dom.boundary_points.shape[0]
    assert np.allclose(flat[bnode], dom.boundary_points)
    assert len(set(bnode.tolist())) == len(bnode)


def test_oracle_solution_is_zero_of_refinement_residual():
    """The refinement drives r = b - J x to zero.  At the oracle's FP64
    solution the leaf rows and the interface flux mismatch vanish."""
    from jaxhps_gb300 import _refinement as rf

    L, p, q = 2, 8, 6
    rng = np.random.default_rng(5)
    root = (-1.0, 1.0, -1.0, 1.0)
    pts = O.leaf_points_2D(O.uniform_leaf_bounds_2D(root, L), p)
    c = 1 + 0.3 * np.sin(pts[..., 0] * 2)
    ones = np.ones_like(c)
    f = rng.standard_normal(pts.shape[:2])
    pr = O.Problem2D(root, L, p, q, {"D_xx": ones, "D_yy": ones, "I": c}, f).build()
    bp = pr.boundary_points
    u = pr.solve(np.cos(bp[:, 0]) * bp[:, 1])
    A = O.assemble_operator(pr.coeffs, pr.ops, 4 ** L, p * p)
    ncb = 4 * (p - 1)
    r1 = f[:, ncb:] - np.einsum("lij,lj->li", A[:, ncb:, :], u)
    assert np.abs(r1).max() < 1e-10 * np.abs(f).max()
    F = np.einsum("ij,lj->li", pr.Q, u)
    nodes = rf.leaf_gauss_nodes_2D(O.uniform_leaf_bounds_2D(root, L), q)
    nbr, _ = rf.node_maps(nodes, bp, scale=2.0)
    Ff = F.reshape(-1)
    inner = nbr >= 0
    assert np.abs(Ff[inner] + Ff[nbr[inner]]).max() < 1e-9 * np.abs(F).max()



def _emulate_merge_iti(Rs, hs, maps):
    """NumPy restatement of the ItI merge gather + Schur complement driven by
    the index maps (what hps_merge_level_iti computes)."""
    Rm, hm = np.stack(Rs), np.stack(hs)
    ni, ne = maps.n_int, maps.n_ext
    oc, pc = maps.int_c[:, 0], maps.int_c[:, 1]
    ol, pl = maps.int_l[:, 0], maps.int_l[:, 1]
    D = np.eye(ni, dtype=complex)
    C = np.zeros((ni, ne), dtype=complex)
    B = np.zeros((ne, ni), dtype=complex)
    A = np.zeros((ne, ne), dtype=complex)
    for u in range(ni):
        for v in range(ni):
            if oc[v] == pc[u]:
                D[u, v] += Rm[pc[u], pl[u], ol[v]]
        for x in range(ne):
            if maps.ext_c[x] == pc[u]:
                C[u, x] = Rm[pc[u], pl[u], maps.ext_l[x]]
    for x in range(ne):
        c, l = maps.ext_c[x], maps.ext_l[x]
        for v in range(ni):
            if oc[v] == c:
                B[x, v] = Rm[c, l, ol[v]]
        for y in range(ne):
            if maps.ext_c[y] == c:
                A[x, y] = Rm[c, l, maps.ext_l[y]]
    dh = hm[pc, pl]
    hext = hm[maps.ext_c, maps.ext_l]
    Dinv = np.linalg.inv(D)
    S = -Dinv @ C
    gt = -Dinv @ dh
    return S, A + B @ S, hext + B @ gt, gt


@pytest.mark.parametrize("nc", [1, 3])
def test_quad_merge_maps_iti_reproduce_oracle(nc):
    rng = np.random.default_rng(11 + nc)
    n = 4 * nc
    Rs = [0.3 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) for _ in range(4)]
    hs = [rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2)) for _ in range(4)]
    S, T, h, gt = O.quad_merge_iti(*Rs, *hs)
    maps = im.quad_merge_maps_iti(nc)
    S2, T2, h2, gt2 = _emulate_merge_iti(Rs, hs, maps)
    assert np.allclose(S, S2) and np.allclose(T, T2) and np.allclose(h, h2) and np.allclose(gt, gt2)
    # the down-pass scatter with the same code reproduces the oracle's ItI propagation
    g = rng.standard_normal((8 * nc, 2)) + 0j
    ref = O._propagate_down_iti(S, g, gt)
    gi = S @ g + gt
    out = np.empty((4, 4 * nc, 2), dtype=complex)
    for c in range(4):
        for k in range(4 * nc):
            cd = maps.code[c, k]
            out[c, k] = g[cd] if cd >= 0 else gi[-cd - 1]
    assert np.allclose(out, ref)


def test_source_upload_falls_back_for_unpinned_sources():
    """The source upload takes the side-stream path only for a page-locked
    CPU tensor of the working dtype bound for a CUDA device; NumPy arrays,
    pageable tensors, other dtypes and CPU targets are converted as before
    (values, shape and the multi-RHS flag unchanged)."""
    import torch
    from jaxhps_gb300 import _stages as st

    rng = np.random.default_rng(0)
    f2 = rng.standard_normal((4, 9))
    f3 = rng.standard_normal((4, 9, 3))
    cpu = torch.device("cpu")
    for src, multi in ((f2, False), (f3, True), (torch.as_tensor(f3), True), (torch.as_tensor(f2, dtype=torch.float32), False)):
        up = st._SourceUpload(src, 4, 9, torch.float64, cpu)
        assert up.out is None and up.event is None
        t, m = up.result()
        assert m is multi
        assert t.dtype == torch.float64 and t.shape == (4, 9, 1 if not multi else 3)
        ref = np.asarray(src, dtype=np.float64)
        np.testing.assert_array_equal(t.numpy(), ref if multi else ref[..., None])


def test_result_copy_into_caller_buffer():
    """solve(out=...) ends in _to_host(out=...): the result is copied into
    the caller's tensor, which is returned; a shape or dtype mismatch is an
    error, not a silent reallocation."""
    import torch
    from jaxhps_gb300 import _stages as st

    t = torch.arange(24, dtype=torch.float64).reshape(2, 3, 4)
    out = torch.zeros(2, 3, 4, dtype=torch.float64)
    r = st._to_host(t, None, out=out)
    assert r is out and torch.equal(out, t)
    with pytest.raises(ValueError):
        st._to_host(t, None, out=torch.zeros(2, 3, 5, dtype=torch.float64))
    with pytest.raises(ValueError):
        st._to_host(t, None, out=torch.zeros(2, 3, 4, dtype=torch.float32))


def test_device_copies_of_fixed_operators_are_made_once():
    """The build's copies of a problem's fixed host operators (P, Q, the
    differential operators) are made once per (key, dtype, device) and
    reused, so a rebuild issues no pageable host-to-device copy."""
    import torch

    from jaxhps_gb300 import _stages as st

    dom = hps.Domain(p=6, q=4, root=hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0), L=1)
    ones = np.ones(dom.interior_points.shape[:2])
    pde = hps.PDEProblem(dom, source=ones, D_xx_coefficients=ones, D_yy_coefficients=ones)
    calls = []

    def make():
        calls.append(1)
        return pde.P

    a = st._device_copy(pde, "P", make, torch.float64, torch.device("cpu"))
    b = st._device_copy(pde, "P", make, torch.float64, torch.device("cpu"))
    c = st._device_copy(pde, "P", make, torch.float32, torch.device("cpu"))
    assert a is b and c is not a and len(calls) == 2
    assert np.array_equal(a.numpy(), pde.P) and c.dtype == torch.float32
    pde.reset()   # dropping the solver state keeps the copies
    assert st._device_copy(pde, "P", make, torch.float64, torch.device("cpu")) is a and len(calls) == 2


def test_pair_kernels_support_table_and_argument_checks_without_a_gpu():
    """Host-only parts of the C ABI: which (p, q) the double-float residual
    kernels are compiled for, and the argument checks of the pair entries,
    which return HPS_ERR_ARG with a message before any device call."""
    import ctypes as C

    from jaxhps_gb300 import _native as nat

    lib = nat.load_library()
    for p in range(4, 20):
        for q in range(2, p):
            want = q == p - 2 and p in (8, 10, 12, 14, 16)
            assert bool(lib.hps_residual_df_supported(p, q)) == want, (p, q)
    null = None
    assert lib.hps_assemble_u_2d_df(0, 16, 14, 1, null, null, null, null, null, null) == 1
    buf = C.create_string_buffer(256)
    lib.hps_last_error(buf, 256)
    assert b"hps_assemble_u_2d_df" in buf.value
    assert lib.hps_mapped_pointer(null, null) == 1

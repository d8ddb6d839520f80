"""GPU implementations of the reference's stage functions.

Each function keeps the reference's name and argument meaning
(local_solve/*.py, merge/*.py, down_pass/*.py) and runs its work through the
native library's C ABI on torch-owned device memory.  Arrays may be given as
NumPy arrays or torch tensors; results are torch tensors on ``device`` (the
solver state is kept in HBM) except the final leaf solutions, which are
moved to ``host_device`` when one is given.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np
import torch

from . import _native as nat
from . import _phases as phases
from ._index_maps import colour_perm, merge_rects, quad_merge_maps_dtn
from ._pdeproblem import COEFF_NAMES_2D, COEFF_NAMES_3D

# Block-structured merge products (merge_rects); HPS_MERGE_RECTS=0 selects the
# dense products.  ItI merges invert D through its two-colour structure
# (colour_perm); HPS_MERGE_TWO_COLOUR=0 inverts D directly.
_RECTS = os.environ.get("HPS_MERGE_RECTS", "1") != "0"
_TWO_COLOUR = os.environ.get("HPS_MERGE_TWO_COLOUR", "1") != "0"


def colour_perm_device(maps, dev):
    perm = colour_perm(maps)
    if perm is None:
        return None
    cache = maps.__dict__.setdefault("_colour_dev", {})
    key = str(dev)
    if key not in cache:
        cache[key] = torch.as_tensor(perm, device=dev)
    return cache[key]

REAL_TO_COMPLEX = {torch.float64: torch.complex128, torch.float32: torch.complex64}

# Device bytes the leaf stage's workspace (the assembled leaf operators) may
# take at once; above it the leaves go in chunks.
LEAF_WORKSPACE_BUDGET = 16 << 30


def _device(device) -> torch.device:
    if device is None or (isinstance(device, str) and device == "cuda"):
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device(device)


def _as_tensor(a, dtype, device) -> torch.Tensor:
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=dtype).contiguous()
    arr = np.asarray(a)
    return torch.as_tensor(np.ascontiguousarray(arr)).to(device=device, dtype=dtype)


def _device_copy(owner, key: str, make, dtype, dev) -> torch.Tensor:
    """Device copy of a small host operator that stays fixed over the life of
    ``owner`` (a PDEProblem's P, Q, G, QH and differential operators), made
    once per (key, dtype, device) and kept on the owner.  A build that reuses
    them issues no pageable host-to-device copy: such a copy blocks the host
    and queues behind an asynchronous source upload on the copy engine, so
    the GPU would idle until that upload ends."""
    cache = owner.__dict__.setdefault("_device_copies", {})
    k = (key, str(dtype), str(dev))
    t = cache.get(k)
    if t is None:
        t = _as_tensor(make(), dtype, dev)
        cache[k] = t
    return t


def _is_complex(a) -> bool:
    if a is None:
        return False
    if isinstance(a, torch.Tensor):
        return a.is_complex()
    return np.iscomplexobj(a)


def _to_host(t: torch.Tensor, host_device, out: torch.Tensor | None = None):
    """``t`` on ``host_device`` (None: left where it is), or copied into
    ``out`` (same shape and dtype) when given.  Device -> CPU copies land in
    page-locked memory (torch caches those blocks), which the copy engines
    fill at full link speed; a pageable destination is staged through a
    bounce buffer at a fraction of it."""
    if out is not None:
        if tuple(out.shape) != tuple(t.shape) or out.dtype != t.dtype:
            raise ValueError(f"out has shape {tuple(out.shape)} and dtype {out.dtype}; the result has "
                             f"shape {tuple(t.shape)} and dtype {t.dtype}")
        out.copy_(t)
        return out
    if host_device is None:
        return t
    dev = torch.device(host_device)
    if dev.type == "cpu" and t.is_cuda:
        out = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        out.copy_(t)
        return out
    return t.to(dev)


def _src3(src, n_leaves, n_pts, dtype, dev):
    """Source as (n_leaves, n_pts, nsrc); returns (tensor, was_multi)."""
    s = _as_tensor(src, dtype, dev)
    if s.dim() == 2:
        return s.unsqueeze(-1).contiguous(), False
    return s, True


class _SourceUpload:
    """The source's host -> device copy, started before the build so that the
    copy engine moves it while the build's kernels run.  A page-locked,
    contiguous CPU tensor of the working dtype is copied on a side stream
    (which first waits for the work already queued on the current stream,
    as the destination block may come from memory that work still uses);
    ``result()`` makes the current stream wait for that copy — a device-side
    wait, the host goes on — and returns (tensor, was_multi) as ``_src3``.
    Any other source is converted by ``_src3`` when ``result()`` is called."""

    def __init__(self, src, n_leaves, n_pts, dtype, dev):
        self.args = (src, n_leaves, n_pts, dtype, dev)
        self.out = None
        self.event = None
        if (isinstance(src, torch.Tensor) and src.device.type == "cpu" and src.dtype == dtype
                and src.is_contiguous() and src.is_pinned() and dev.type == "cuda"):
            main = torch.cuda.current_stream(dev)
            side = torch.cuda.Stream(device=dev)
            dst = torch.empty(src.shape, dtype=dtype, device=dev)
            side.wait_stream(main)
            timed = phases.enabled()
            with torch.cuda.stream(side):
                if timed:
                    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    t0.record()
                dst.copy_(src, non_blocking=True)
                if timed:
                    t1.record()
                    phases.side("source_h2d", t0, t1)
            dst.record_stream(side)   # the block is not reused before the copy ends, even if the build fails
            self.event = torch.cuda.Event()
            self.event.record(side)
            self.out = dst

    def result(self):
        if self.out is None:
            return _src3(*self.args)
        src, n_leaves, n_pts, dtype, dev = self.args
        torch.cuda.current_stream(dev).wait_event(self.event)
        s = self.out
        if s.dim() == 2:
            return s.unsqueeze(-1), False
        return s, True


def _coefficients(pde_problem, dev):
    cs, ops = pde_problem.active_coefficients()
    if not cs:
        raise ValueError("PDEProblem has no differential operator coefficients")
    cplx = any(_is_complex(c) for c in cs)
    ctype = torch.complex128 if cplx else torch.float64
    coeffs = torch.stack([_as_tensor(c, ctype, dev) for c in cs]).contiguous()
    names = tuple(n for n in (COEFF_NAMES_2D if pde_problem.domain.bool_2D else COEFF_NAMES_3D)
                  if getattr(pde_problem, f"{n}_coefficients") is not None)
    ops_t = _device_copy(pde_problem, "ops:" + ",".join(names), lambda: np.stack(ops), torch.float64, dev)
    phases.mark("coefficients_h2d")
    return ops_t, coeffs, cplx


# ---------------------------------------------------------------------------
# Leaf stage
# ---------------------------------------------------------------------------


def local_solve_stage_uniform_2D_DtN(pde_problem, host_device=None, device=None, dtype=torch.float64,
                                     keep_inverse: bool = False):
    """Leaf DtN solve for every leaf (reference local_solve/_uniform_2D_DtN.py:9-102).

    Returns ``(Y, T, v, h)``: Y (n_leaves, p^2, 4q), T (n_leaves, 4q, 4q),
    v (n_leaves, p^2[, nsrc]), h (n_leaves, 4q[, nsrc]).  With
    ``keep_inverse`` the per-leaf ``inv(A_ii)`` is returned as a fifth item.
    """
    return _local_solve_dtn(pde_problem, pde_problem.P, pde_problem.Q, device, dtype, keep_inverse)


@phases.ranged("leaf solve (DtN)")
def _local_solve_dtn(pde_problem, P_np, Q_np, device, dtype, keep_inverse, source=None, want_source=True,
                     coefficients=None):
    """``coefficients`` = (ops, coeffs, is_complex) overrides the problem's own
    (adaptive leaves pass per-leaf rescaled coefficients)."""
    L = nat.lib()
    dev = _device(device)
    dom = pde_problem.domain
    n_leaves = dom.n_leaves
    n_pts = dom.interior_points.shape[1]
    n_cb = P_np.shape[0]
    ng = P_np.shape[1]
    ops_t, coeffs, cplx = _coefficients(pde_problem, dev) if coefficients is None else coefficients
    if cplx or _is_complex(pde_problem.source if source is None else source):
        dtype = REAL_TO_COMPLEX.get(dtype, dtype)
    P = _device_copy(pde_problem, "P", lambda: P_np, dtype, dev) if P_np is pde_problem.P else \
        _as_tensor(P_np, dtype, dev)
    Q = _device_copy(pde_problem, "Q", lambda: Q_np, dtype, dev) if Q_np is pde_problem.Q else \
        _as_tensor(Q_np, dtype, dev)
    src = pde_problem.source if source is None else source
    multi = False
    if want_source and src is not None:
        f, multi = _src3(src, n_leaves, n_pts, dtype, dev)
        ns = f.shape[-1]
    else:
        f, ns = None, 0
    n_i = n_pts - n_cb
    Y = torch.empty((n_leaves, n_pts, ng), dtype=dtype, device=dev)
    T = torch.empty((n_leaves, ng, ng), dtype=dtype, device=dev)
    v = torch.empty((n_leaves, n_pts, ns), dtype=dtype, device=dev) if ns else None
    h = torch.empty((n_leaves, ng, ns), dtype=dtype, device=dev) if ns else None
    Aii = torch.empty((n_leaves, n_i, n_i), dtype=dtype, device=dev)
    info = torch.zeros(n_leaves, dtype=torch.int32, device=dev)
    a = nat.LeafDtnArgs(
        dtype=nat.TORCH_TO_HPS[dtype], coef_complex=int(cplx), n_leaves=n_leaves, n_pts=n_pts, n_cb=n_cb,
        n_gauss=ng, nsrc=ns, n_ops=ops_t.shape[0], ops=ops_t.data_ptr(), coeffs=coeffs.data_ptr(),
        source=nat.ptr(f), P=P.data_ptr(), Q=Q.data_ptr(), Y=Y.data_ptr(), T=T.data_ptr(), v=nat.ptr(v),
        h=nat.ptr(h), Aii_inv=Aii.data_ptr(), info=info.data_ptr(), workspace=None, workspace_bytes=0)
    wsb = L.hps_local_solve_dtn_workspace_size(C.byref(a))
    if wsb <= LEAF_WORKSPACE_BUDGET or n_leaves == 1:
        ws = nat.workspace(wsb, dev)
        a.workspace, a.workspace_bytes = ws.data_ptr(), ws.numel()
        nat.check(L.hps_local_solve_dtn(C.byref(a), nat.stream_ptr()), "hps_local_solve_dtn")
    else:
        # the assembled leaf operators of every leaf would not fit the budget:
        # leaves in chunks (the reference chunks its leaf stage as well,
        # _device_config.py:65-90), one workspace reused by all chunks
        chunk = max(1, int(n_leaves * LEAF_WORKSPACE_BUDGET // wsb))
        es = torch.empty((), dtype=dtype).element_size()
        for lo in range(0, n_leaves, chunk):
            hi = min(n_leaves, lo + chunk)
            cc = coeffs[:, lo:hi].contiguous()
            b = nat.LeafDtnArgs(
                dtype=a.dtype, coef_complex=a.coef_complex, n_leaves=hi - lo, n_pts=n_pts, n_cb=n_cb, n_gauss=ng,
                nsrc=ns, n_ops=a.n_ops, ops=a.ops, coeffs=cc.data_ptr(),
                source=None if f is None else f.data_ptr() + lo * n_pts * ns * es, P=a.P, Q=a.Q,
                Y=Y.data_ptr() + lo * n_pts * ng * es, T=T.data_ptr() + lo * ng * ng * es,
                v=None if v is None else v.data_ptr() + lo * n_pts * ns * es,
                h=None if h is None else h.data_ptr() + lo * ng * ns * es,
                Aii_inv=Aii.data_ptr() + lo * n_i * n_i * es, info=info.data_ptr() + lo * 4, workspace=None,
                workspace_bytes=0)
            wsc = L.hps_local_solve_dtn_workspace_size(C.byref(b))
            ws = nat.workspace(wsc, dev)
            b.workspace, b.workspace_bytes = ws.data_ptr(), ws.numel()
            nat.check(L.hps_local_solve_dtn(C.byref(b), nat.stream_ptr()), "hps_local_solve_dtn")
            del cc
    if v is not None and not multi:
        v, h = v[..., 0], h[..., 0]
    out = (Y, T, v, h)
    if keep_inverse:
        out = out + (Aii,)
    pde_problem._leaf_info = info
    return out


def local_solve_stage_uniform_3D_DtN(pde_problem, host_device=None, device=None, dtype=torch.float64,
                                     keep_inverse: bool = False):
    """Leaf DtN solve for 3D leaves (reference local_solve/_uniform_3D_DtN.py:13-106);
    the leaf algebra is the same as 2D with p^3 points and 6q^2 Gauss nodes."""
    return _local_solve_dtn(pde_problem, pde_problem.P, pde_problem.Q, device, dtype, keep_inverse)


@phases.ranged("leaf solve (ItI)")
def local_solve_stage_uniform_2D_ItI(pde_problem, host_device=None, device=None, dtype=torch.complex128,
                                     keep_inverse: bool = False):
    """Leaf ItI solve (reference local_solve/_uniform_2D_ItI.py:10-186).

    Returns ``(Y, T, v, h)`` with T the impedance-to-impedance map."""
    L = nat.lib()
    dev = _device(device)
    dom = pde_problem.domain
    n_leaves = dom.n_leaves
    n_pts = dom.interior_points.shape[1]
    P_np = pde_problem.P
    n_cb, ng = P_np.shape
    ops_t, coeffs, cplx = _coefficients(pde_problem, dev)
    dtype = REAL_TO_COMPLEX.get(dtype, dtype)
    P = _device_copy(pde_problem, "P", lambda: P_np, dtype, dev)
    G = _device_copy(pde_problem, "G", lambda: pde_problem.G, dtype, dev)
    QH = _device_copy(pde_problem, "QH", lambda: pde_problem.QH, dtype, dev)
    multi = False
    if pde_problem.source is not None:
        f, multi = _src3(pde_problem.source, n_leaves, n_pts, dtype, dev)
        ns = f.shape[-1]
    else:
        f, ns = None, 0
    Y = torch.empty((n_leaves, n_pts, ng), dtype=dtype, device=dev)
    T = torch.empty((n_leaves, ng, ng), dtype=dtype, device=dev)
    v = torch.empty((n_leaves, n_pts, ns), dtype=dtype, device=dev) if ns else None
    h = torch.empty((n_leaves, ng, ns), dtype=dtype, device=dev) if ns else None
    Binv = torch.empty((n_leaves, n_pts, n_pts), dtype=dtype, device=dev)
    info = torch.zeros(n_leaves, dtype=torch.int32, device=dev)
    a = nat.LeafItiArgs(
        dtype=nat.TORCH_TO_HPS[dtype], coef_complex=int(cplx), n_leaves=n_leaves, n_pts=n_pts, n_cb=n_cb,
        n_gauss=ng, nsrc=ns, n_ops=ops_t.shape[0], ops=ops_t.data_ptr(), coeffs=coeffs.data_ptr(),
        source=nat.ptr(f), G=G.data_ptr(), P=P.data_ptr(), QH=QH.data_ptr(), Y=Y.data_ptr(), T=T.data_ptr(),
        v=nat.ptr(v), h=nat.ptr(h), B_inv=Binv.data_ptr(), info=info.data_ptr(), workspace=None,
        workspace_bytes=0)
    wsb = L.hps_local_solve_iti_workspace_size(C.byref(a))
    ws = nat.workspace(wsb, dev)
    a.workspace, a.workspace_bytes = ws.data_ptr(), ws.numel()
    nat.check(L.hps_local_solve_iti(C.byref(a), nat.stream_ptr()), "hps_local_solve_iti")
    if v is not None and not multi:
        v, h = v[..., 0], h[..., 0]
    out = (Y, T, v, h)
    if keep_inverse:
        out = out + (Binv,)
    pde_problem._leaf_info = info
    return out


# ---------------------------------------------------------------------------
# Merge stage
# ---------------------------------------------------------------------------


def check_infos(infos, what: str = "batched inverse") -> None:
    """Status words of batched inverses: -1 marks a matrix whose multi-CTA
    panel barrier timed out (its result is invalid), k > 0 an exactly zero
    pivot at column k (the matrix is singular).  One device sync for all."""
    infos = [i for i in (infos or []) if i is not None and i.numel()]
    if not infos:
        return
    lo, hi = (int(x) for x in torch.stack([torch.stack([i.min(), i.max()]) for i in infos]).aminmax())
    if lo < 0:
        raise nat.DeviceWaitTimeout(f"{what}: a multi-CTA panel barrier timed out; results are invalid")
    if hi > 0:
        bad = next(i for i in infos if int(i.max()) > 0)
        m = int(torch.nonzero(bad > 0)[0, 0])
        raise nat.SingularPivotError(f"{what}: matrix {m} of a batch is singular (zero pivot at column "
                                     f"{int(bad[m]) - 1})")


def raise_on_sync_timeout(infos) -> None:
    """check_infos for the merge inverses (kept name)."""
    check_infos(infos, "merge inverse")


@phases.ranged("merge level")
def merge_level_dtn(T_children: torch.Tensor, h_children, maps, keep_D_inv=False, keep_BD_inv=False,
                    keep_B=False, iti=False, need_T=True, infos=None):
    """One batched merge level.  T_children: (n_merges*nch, nb, nb);
    h_children: (n_merges*nch, nb, nsrc) or None.  Returns
    (S, g_tilde, T_out, h_out, D_inv, BD_inv) and B when ``keep_B``.
    With ``need_T=False`` the merged map is not formed (T_out is None)."""
    L = nat.lib()
    dev = T_children.device
    dtype = T_children.dtype
    nch, nb, n_int, n_ext = maps.nch, maps.nb, maps.n_int, maps.n_ext
    assert T_children.shape[1] == nb and T_children.shape[0] % nch == 0
    n_m = T_children.shape[0] // nch
    ns = 0 if h_children is None else h_children.shape[-1]
    S = torch.empty((n_m, n_int, n_ext), dtype=dtype, device=dev)
    T_out = torch.empty((n_m, n_ext, n_ext), dtype=dtype, device=dev) if need_T else None
    g_t = torch.empty((n_m, n_int, ns), dtype=dtype, device=dev) if ns else None
    h_out = torch.empty((n_m, n_ext, ns), dtype=dtype, device=dev) if ns else None
    D_inv = torch.empty((n_m, n_int, n_int), dtype=dtype, device=dev) if keep_D_inv else None
    BD_inv = torch.empty((n_m, n_ext, n_int), dtype=dtype, device=dev) if keep_BD_inv else None
    B = torch.empty((n_m, n_ext, n_int), dtype=dtype, device=dev) if keep_B else None
    info = torch.zeros(n_m, dtype=torch.int32, device=dev)
    md = maps.device(dev)
    a = nat.MergeArgs(
        dtype=nat.TORCH_TO_HPS[dtype], n_merges=n_m, nch=nch, nb=nb, n_int=n_int, n_ext=n_ext, nsrc=ns,
        T_children=T_children.data_ptr(), h_children=nat.ptr(h_children), int_c=md["int_c"].data_ptr(),
        int_l=md["int_l"].data_ptr(), ext_c=md["ext_c"].data_ptr(), ext_l=md["ext_l"].data_ptr(),
        loc=md["loc"].data_ptr(), S=S.data_ptr(), g_tilde=nat.ptr(g_t), T_out=nat.ptr(T_out),
        h_out=nat.ptr(h_out), D_inv=nat.ptr(D_inv), BD_inv=nat.ptr(BD_inv), B_out=nat.ptr(B),
        info=info.data_ptr(), workspace=None, workspace_bytes=0)
    rects = merge_rects(maps, iti) if _RECTS else None
    if rects is not None:
        a.n_c_rects, a.c_rects = rects[0].shape[0], rects[0].ctypes.data
        a.n_b_rects, a.b_rects = rects[1].shape[0], rects[1].ctypes.data
    if iti and _TWO_COLOUR:
        cp = colour_perm_device(maps, dev)
        if cp is not None:
            a.n_x, a.colour_perm = n_int // 2, cp.data_ptr()
    wsb = L.hps_merge_level_dtn_workspace_size(C.byref(a))
    ws = nat.workspace(wsb, dev)
    a.workspace, a.workspace_bytes = ws.data_ptr(), ws.numel()
    if iti:
        nat.check(L.hps_merge_level_iti(C.byref(a), nat.stream_ptr()), "hps_merge_level_iti")
    else:
        nat.check(L.hps_merge_level_dtn(C.byref(a), nat.stream_ptr()), "hps_merge_level_dtn")
    if infos is not None:
        infos.append(info)
    if keep_B:
        return S, g_t, T_out, h_out, D_inv, BD_inv, B
    return S, g_t, T_out, h_out, D_inv, BD_inv


@phases.ranged("up level")
def up_level(h_children, D_inv, B, maps, b_is_bd_inv: bool = False, iti: bool = False):
    """One up-pass level with stored D_inv and B, or B D_inv with
    ``b_is_bd_inv`` (reference up_pass/_uniform_2D_DtN.py:8-173,
    up_pass/_uniform_2D_ItI.py:8-214): returns (g_tilde, h_out)."""
    L = nat.lib()
    n_m, n_int, _ = D_inv.shape
    n_ext = B.shape[1]
    ns = h_children.shape[-1]
    dev, dtype = D_inv.device, D_inv.dtype
    dh = torch.empty((n_m, n_int, ns), dtype=dtype, device=dev)
    g_t = torch.empty((n_m, n_int, ns), dtype=dtype, device=dev)
    h_out = torch.empty((n_m, n_ext, ns), dtype=dtype, device=dev)
    md = maps.device(dev)
    a = nat.UpArgs(dtype=nat.TORCH_TO_HPS[dtype], n_merges=n_m, nch=maps.nch, nb=maps.nb, n_int=n_int, n_ext=n_ext,
                   nsrc=ns, h_children=h_children.data_ptr(), int_c=md["int_c"].data_ptr(),
                   int_l=md["int_l"].data_ptr(), ext_c=md["ext_c"].data_ptr(), ext_l=md["ext_l"].data_ptr(),
                   D_inv=D_inv.data_ptr(), B=B.data_ptr(), dh=dh.data_ptr(), g_tilde=g_t.data_ptr(),
                   h_out=h_out.data_ptr(),
                   flags=(nat.HPS_UP_B_IS_BD_INV if b_is_bd_inv else 0) | (nat.HPS_UP_ITI if iti else 0))
    nat.check(L.hps_up_level(C.byref(a), nat.stream_ptr()), "hps_up_level")
    return g_t, h_out


def merge_stage_generic(T_arr, h_arr, n_levels: int, maps_fn, device=None, subtree_recomp: bool = False,
                        return_T: bool = False, keep_D_inv: bool = False):
    """Level loop shared by the quad and oct DtN merge stages.  ``maps_fn(nb)``
    gives the merge maps for children with ``nb`` boundary points.  The top
    level's merged map is formed only when it is returned."""
    dev = _device(device)
    T = T_arr if isinstance(T_arr, torch.Tensor) else _as_tensor(T_arr, torch.float64, dev)
    T = T.to(dev).contiguous()
    if T.dim() == 4:
        T = T.reshape(-1, T.shape[-2], T.shape[-1])
    multi = h_arr is not None and np.ndim(h_arr) == 3 if not isinstance(h_arr, torch.Tensor) else (
        h_arr is not None and h_arr.dim() == 3)
    h = None
    if h_arr is not None:
        h = h_arr if isinstance(h_arr, torch.Tensor) else _as_tensor(h_arr, T.dtype, dev)
        h = h.to(device=dev, dtype=T.dtype)
        if h.dim() == 2:
            h = h.unsqueeze(-1)
        h = h.reshape(T.shape[0], T.shape[1], -1).contiguous()
    S_lst, g_lst, Dinv_lst, infos = [], [], [], []
    for lvl in range(n_levels):
        maps = maps_fn(T.shape[1])
        need_T = lvl < n_levels - 1 or return_T or subtree_recomp
        S, g_t, T, h, D_inv, _ = merge_level_dtn(T, h, maps, keep_D_inv=keep_D_inv, need_T=need_T, infos=infos)
        S_lst.append(S)
        g_lst.append(g_t if (g_t is None or multi) else g_t[..., 0])
        Dinv_lst.append(D_inv)
    raise_on_sync_timeout(infos)
    if subtree_recomp:
        return T, (h if (h is None or multi) else h[..., 0])
    out = (S_lst, g_lst)
    if return_T:
        out = out + (T[0],)
    if keep_D_inv:
        out = out + (Dinv_lst,)
    return out


def merge_stage_uniform_2D_DtN(T_arr, h_arr, l: int, device=None, host_device=None, subtree_recomp: bool = False,
                               return_T: bool = False, keep_D_inv: bool = False):
    """Level loop of DtN quad merges (reference merge/_uniform_2D_DtN.py:13-203).

    Returns ``(S_lst, g_tilde_lst)`` (leaf-adjacent level first, root last,
    root with a leading batch axis of 1) and the top-level T when
    ``return_T``.  With ``subtree_recomp`` returns only the top ``(T, h)``.
    """
    return merge_stage_generic(T_arr, h_arr, max(int(l), 1), lambda nb: quad_merge_maps_dtn(nb // 4), device,
                               subtree_recomp, return_T, keep_D_inv)


# ---------------------------------------------------------------------------
# Down pass
# ---------------------------------------------------------------------------


@phases.ranged("down level")
def down_level(S, g_tilde, g_parent, maps):
    """One level of boundary-data propagation (n_merges parents -> nch*n_merges children)."""
    L = nat.lib()
    n_m, n_int, n_ext = S.shape
    ns = g_parent.shape[-1]
    dev, dtype = S.device, S.dtype
    g_int = torch.empty((n_m, n_int, ns), dtype=dtype, device=dev)
    g_ch = torch.empty((n_m * maps.nch, maps.nb, ns), dtype=dtype, device=dev)
    md = maps.device(dev)
    a = nat.DownArgs(dtype=nat.TORCH_TO_HPS[dtype], n_merges=n_m, nch=maps.nch, nb=maps.nb, n_int=n_int,
                     n_ext=n_ext, nsrc=ns, S=S.data_ptr(), g_tilde=nat.ptr(g_tilde), g_parent=g_parent.data_ptr(),
                     code=md["code"].data_ptr(), g_int=g_int.data_ptr(), g_children=g_ch.data_ptr())
    nat.check(L.hps_down_level(C.byref(a), nat.stream_ptr()), "hps_down_level")
    return g_ch


def _down_pass_generic(boundary_data, S_lst, g_tilde_lst, Y_arr, v_arr, maps_fn, device, host_device,
                       ext_per_unit: int = 8):
    """Down pass over the stored levels; ``maps_fn(n)`` gives the merge maps of
    a level whose parents have ``ext_per_unit * n`` exterior points (8nc in
    2D, 24nf in 3D)."""
    dev = _device(device)
    dtype = S_lst[0].dtype
    g = boundary_data if isinstance(boundary_data, torch.Tensor) else _as_tensor(boundary_data, dtype, dev)
    g = g.to(device=dev, dtype=dtype)
    multi_g = g_tilde_lst[0] is not None and g_tilde_lst[0].dim() == 3
    if g.dim() == 1:
        g = g.unsqueeze(-1)
    if g.dim() == 2:
        g = g.unsqueeze(0)
    g = g.contiguous()
    ns = g.shape[-1]
    for lvl in range(len(S_lst) - 1, -1, -1):
        S = S_lst[lvl]
        gt = g_tilde_lst[lvl]
        if gt is not None and gt.dim() == 2:
            gt = gt.unsqueeze(-1)
        if gt is not None and gt.shape[-1] != ns:
            if gt.shape[-1] == 1:
                gt = gt.expand(-1, -1, ns)
            else:
                raise ValueError("boundary data and g_tilde have different numbers of sources")
        gt = None if gt is None else gt.contiguous()
        nc_child = S.shape[2] // ext_per_unit
        g = down_level(S, gt, g, maps_fn(nc_child))
    if Y_arr is None:
        return g if (ns > 1 or multi_g) else g[..., 0]
    u = torch.empty((Y_arr.shape[0], Y_arr.shape[1], ns), dtype=dtype, device=dev)
    if v_arr is not None:
        v = v_arr if v_arr.dim() == 3 else v_arr.unsqueeze(-1)
        if v.shape[-1] != ns:
            v = v.expand(-1, -1, ns)
        v = v.contiguous()
        nat.gemm(Y_arr, g, u, 1.0, 1.0, Cmat=v)
    else:
        nat.gemm(Y_arr, g, u)
    if ns == 1 and not multi_g and (v_arr is None or v_arr.dim() == 2):
        u = u[..., 0]
    return _to_host(u, host_device)


def down_pass_uniform_2D_DtN(boundary_data, S_lst, g_tilde_lst, Y_arr, v_arr, device=None, host_device=None):
    """Reference down_pass/_uniform_2D_DtN.py:7-122.  If ``Y_arr`` is None the
    leaf boundary data is returned instead of the leaf solutions."""
    return _down_pass_generic(boundary_data, S_lst, g_tilde_lst, Y_arr, v_arr, quad_merge_maps_dtn, device,
                              host_device)

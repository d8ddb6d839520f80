"""Mixed-precision ItI (Helmholtz-type) build and refined solve, uniform 2D.

Build (complex64): the leaf inverses inv(B), B = [G; A_int] (the reference's
get_ItI, local_solve/_uniform_2D_ItI.py:120-186), the leaf maps Y, and per
merge level S, D^-1 and B D^-1 (merge/_uniform_2D_ItI.py with the no-source
bookkeeping of merge/_nosource_uniform_2D_ItI.py) — a complex64 HPS solver
used as the approximate inverse M.  Each leaf's interior rows A_int are
assembled once in complex128 for the residuals.

Solve: unknowns u (every leaf point) and t (incoming impedance at every leaf
Gauss node), complex128, from zero.  The discrete system J is
    leaf rows       B u = [P t ; f_int]
    interface rows  t(a) + t_out(b) = 0  at paired nodes a, b  (t_out = QH u)
    boundary rows   t = given incoming impedance data
and each iteration computes its residual in complex128 (hps_residual_iti_2d:
tensor-product derivatives, no stored per-leaf rows) and applies M:
    v  = inv(B) r_leaf,  h = QH v + hcorr  (hcorr: the interface residuals),
    up pass with D^-1, B D^-1; down pass from the boundary residual -> dt,
    du = Y dt + v;  u += du, t += dt
until the remaining error is at most tol max|u| (``_refinement.converged``).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import List

import ctypes as C

import numpy as np
import torch

from . import _native as nat
from . import _stages as st
from ._index_maps import quad_merge_maps_iti
from ._nosource import _nosource_merge, store_operators
from ._pdeproblem import COEFF_NAMES_2D
from ._refinement import OP_KIND_2D, _domain_constants, converged, raise_not_converged
from ._refinement_dense import _node_pairing


@dataclass
class ItiMixedState:
    mixed: bool
    iti: bool
    n_leaves: int
    n_pts: int
    n_cb: int
    p: int
    q: int
    eta: float
    coeffs: torch.Tensor        # (n_ops, n_leaves, p^2) float64 or complex128
    op_kind: List[int]
    consts: dict
    Binv: torch.Tensor          # (n_leaves, n_pts, n_pts) complex64
    Y: torch.Tensor             # (n_leaves, n_pts, n_g) complex64
    QH32: torch.Tensor          # (n_g, n_pts) complex64
    S_lst: List[torch.Tensor]
    Dinv_lst: List[torch.Tensor]
    BDinv_lst: List[torch.Tensor]
    f: torch.Tensor             # (n_leaves, n_pts, nsrc) complex128
    multi: bool
    nbr: torch.Tensor
    bnode: torch.Tensor
    tol: float = 1e-12
    max_iters: int = 30
    history: list = field(default_factory=list)


def _coefficients(pde_problem, dev):
    """Active coefficients stacked (n_ops, n_leaves, p^2) and their op kinds;
    complex128 when any coefficient is complex."""
    arrs, names = [], []
    for name in COEFF_NAMES_2D:
        c = getattr(pde_problem, f"{name}_coefficients")
        if c is not None:
            arrs.append(c)
            names.append(name)
    cplx = any(st._is_complex(c) for c in arrs)
    dt = torch.complex128 if cplx else torch.float64
    return torch.stack([st._as_tensor(c, dt, dev) for c in arrs]).contiguous(), [OP_KIND_2D[n] for n in names]


def build_mixed_iti(pde_problem, return_top_T=False, device=None, tol: float = 1e-12, max_iters: int = 30):
    dom = pde_problem.domain
    if not pde_problem.use_ItI or not dom.bool_2D or not dom.bool_uniform:
        raise NotImplementedError("this mixed-precision path serves uniform 2D ItI problems")
    if pde_problem.source is None:
        raise ValueError("mixed precision needs the source at build time")
    r = dom.root
    if not np.isclose(r.xmax - r.xmin, r.ymax - r.ymin):
        raise NotImplementedError("the mixed-precision residual assumes square leaves")
    dev = st._device(device)
    src = pde_problem.source
    upload = st._SourceUpload(src, dom.n_leaves, pde_problem.G.shape[1], torch.complex128, dev)
    pde_problem.source = None
    try:
        Y, T, _, _, Binv = st.local_solve_stage_uniform_2D_ItI(pde_problem, device=dev, dtype=torch.complex64,
                                                               keep_inverse=True)
    finally:
        pde_problem.source = src
    n_cb, n_pts = pde_problem.G.shape
    nl = dom.n_leaves
    coeffs, op_kind = _coefficients(pde_problem, dev)
    out = _nosource_merge(T, dom.L, True, dev, return_top_T)
    del T
    f, multi = upload.result()
    nbr, bnode = _node_pairing(dom, dev)
    QH32 = torch.as_tensor(np.ascontiguousarray(pde_problem.QH), device=dev).to(torch.complex64)
    state = ItiMixedState(
        mixed=True, iti=True, n_leaves=nl, n_pts=n_pts, n_cb=n_cb, p=dom.p, q=dom.q, eta=float(pde_problem.eta),
        coeffs=coeffs, op_kind=op_kind, consts=_domain_constants(dom, dev), Binv=Binv, Y=Y, QH32=QH32,
        S_lst=out[0], Dinv_lst=out[1], BDinv_lst=out[2], f=f, multi=multi, nbr=nbr, bnode=bnode, tol=tol,
        max_iters=max_iters)
    pde_problem._state = state
    pde_problem._precision = "mixed"
    pde_problem.Y = Y
    pde_problem.S_lst = out[0]
    store_operators(pde_problem, out[1], out[2], True)
    pde_problem.g_tilde_lst = []
    if return_top_T:
        return out[3]
    return None


def _residual(state: ItiMixedState, u, t, r32, t_out):
    """r32 = [P t - G u ; f_int - A_int u] per leaf (complex64), t_out = QH u
    (complex128), both from complex128 arithmetic."""
    cs = state.consts
    a = nat.ResidualIti2DArgs(
        n_leaves=state.n_leaves, p=state.p, q=state.q, nsrc=u.shape[-1], n_ops=len(state.op_kind),
        coef_complex=int(state.coeffs.is_complex()), eta=state.eta, coeffs=state.coeffs.data_ptr(),
        inv_half=cs["inv_half"].data_ptr(), D1=cs["D1"].data_ptr(), D2=cs["D2"].data_ptr(),
        Pside=cs["Pside"].data_ptr(), Qside=cs["Qside"].data_ptr(), perm=cs["perm"].data_ptr(), u=u.data_ptr(),
        t_in=t.data_ptr(), f=state.f.data_ptr(), r=r32.data_ptr(), t_out=t_out.data_ptr())
    for i, k in enumerate(state.op_kind):
        a.op_kind[i] = k
    nat.check(nat.lib().hps_residual_iti_2d(C.byref(a), nat.stream_ptr()), "hps_residual_iti_2d")


def correction(state: ItiMixedState, r32, hcorr, rb32):
    """(du, dt) = M r with the complex64 operators."""
    v = torch.empty_like(r32)
    nat.gemm(state.Binv, r32, v)
    h = torch.empty_like(hcorr)
    nat.gemm(state.QH32, v, h, 1.0, 1.0, Cmat=hcorr)
    g_t_lst = []
    for Dinv, BDinv in zip(state.Dinv_lst, state.BDinv_lst):
        g_t, h = st.up_level(h, Dinv, BDinv, quad_merge_maps_iti(BDinv.shape[1] // 8), b_is_bd_inv=True, iti=True)
        g_t_lst.append(g_t)
    gch = rb32.unsqueeze(0)
    for lvl in range(len(state.S_lst) - 1, -1, -1):
        S = state.S_lst[lvl]
        gch = st.down_level(S, g_t_lst[lvl], gch, quad_merge_maps_iti(S.shape[2] // 8))
    nat.gemm(state.Y, gch, v, 1.0, 1.0, Cmat=v)     # du = Y dt + v
    return v, gch


def _accumulate(x32: torch.Tensor, y64: torch.Tensor) -> None:
    """y64 += x32 for complex tensors (as interleaved real pairs)."""
    nat.check(nat.lib().hps_accumulate(2 * x32.numel(), x32.data_ptr(), y64.data_ptr(), nat.stream_ptr()),
              "hps_accumulate")


def solve_mixed_iti(pde_problem, boundary_data, source=None, host_device="cpu", tol=None, max_iters=None):
    state: ItiMixedState = pde_problem._state
    if source is not None:
        raise ValueError("the mixed-precision solver takes the source at build time")
    L = nat.lib()
    dev = state.Binv.device
    tol = state.tol if tol is None else tol
    max_iters = state.max_iters if max_iters is None else max_iters
    ns = state.f.shape[-1]
    tg = boundary_data if isinstance(boundary_data, torch.Tensor) else torch.as_tensor(np.asarray(boundary_data))
    tg = tg.to(device=dev, dtype=torch.complex128)
    if tg.dim() == 1:
        tg = tg.unsqueeze(-1)
    if tg.shape[-1] != ns:
        if tg.shape[-1] == 1:
            tg = tg.expand(-1, ns)
        else:
            raise ValueError("boundary data and source have different numbers of right-hand sides")
    tg = tg.contiguous()
    nl, n_pts = state.n_leaves, state.n_pts
    ng = state.Y.shape[2]
    u = torch.zeros((nl, n_pts, ns), dtype=torch.complex128, device=dev)
    t = torch.zeros((nl, ng, ns), dtype=torch.complex128, device=dev)
    t_out = torch.zeros((nl, ng, ns), dtype=torch.complex128, device=dev)
    r32 = torch.empty((nl, n_pts, ns), dtype=torch.complex64, device=dev)
    hcorr = torch.empty((nl, ng, ns), dtype=torch.complex64, device=dev)
    rb32 = torch.empty((tg.shape[0], ns), dtype=torch.complex64, device=dev)
    sp = nat.stream_ptr()
    _residual(state, u, t, r32, t_out)
    maxima = torch.empty(2, dtype=torch.float64, device=dev)
    state.history = []
    for _ in range(max_iters):
        nat.check(L.hps_iti_combine(nl * ng, ns, state.nbr.data_ptr(), t_out.data_ptr(), t.data_ptr(), hcorr.data_ptr(),
                                    tg.shape[0], state.bnode.data_ptr(), tg.data_ptr(), rb32.data_ptr(), sp),
                  "hps_iti_combine")
        du, dt = correction(state, r32, hcorr, rb32)
        _accumulate(dt, t)
        step, size = nat.accumulate_max(du, u, maxima, pairs=True)
        state.history.append(step / max(size, 1e-300))
        if converged(state.history, tol):
            break
        _residual(state, u, t, r32, t_out)
    else:
        raise_not_converged(state.history, tol, max_iters, "mixed-precision ItI solve")
    nat.raise_on_tc_timeout("mixed-precision ItI solve")
    if not state.multi:
        u = u[..., 0]
    return st._to_host(u, host_device)

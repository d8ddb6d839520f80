"""Mixed-precision build and iteratively refined solve for uniform DtN trees
of either dimension, with FP64 residuals evaluated from each leaf's
assembled interior operator rows (used for 3D octrees; the 2D quadtree path
in ``_refinement`` evaluates the same residual with tensor-product kernels).

Build (FP32): leaf inverses inv(A_ii), the interior rows of Y (refined once
against FP64 residuals), and for every merge level S, inv(D) and B — a
complete FP32 HPS direct solver used as an approximate inverse M of the
discrete system J.  The interior rows A_int = A[n_cb:, :] of every leaf are
assembled once in FP64 (hps_assemble_rows) and kept for the residuals.

Solve: x = (u_int, g) in FP64 from zero, iterating r = b - J x (FP64
strided GEMMs), dx = M r (FP32 leaf inverse, up pass, down pass), x += dx,
until the remaining error is at most tol * max|u|
(``_refinement.converged``).  J is the system the reference's FP64 direct
solver solves exactly: leaf collocation rows (local_solve/_uniform_3D_DtN.py
:13-106 with get_DtN, local_solve/_uniform_2D_DtN.py:228-273), continuity
of the outward normal derivative across interfaces (the merge equations,
merge/_schur_complement.py:182-237, :293-774) and the Dirichlet data on the
domain boundary.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, List

import numpy as np
import torch

from . import _native as nat
from . import _stages as st
from ._index_maps import oct_merge_maps_dtn, quad_merge_maps_dtn
from ._refinement import converged, leaf_gauss_nodes_2D, node_maps, raise_not_converged


def _maps_for_ext(dim: int) -> Callable:
    """Merge maps of a level from its parents' exterior size."""
    if dim == 2:
        return lambda n_ext: quad_merge_maps_dtn(n_ext // 8)
    return lambda n_ext: oct_merge_maps_dtn(n_ext // 24)


@dataclass
class DenseMixedState:
    mixed: bool
    dense: bool
    dim: int
    n_leaves: int
    n_pts: int
    n_cb: int
    Aint: torch.Tensor           # (n_leaves, n_i, n_pts) FP64 interior operator rows
    P64: torch.Tensor            # (n_cb, n_g) FP64
    Q64: torch.Tensor            # (n_g, n_pts) FP64
    Y_int: torch.Tensor          # (n_leaves, n_i, n_g) FP32 view
    Aii_inv: torch.Tensor        # (n_leaves, n_i, n_i) FP32
    Q_int: torch.Tensor          # (n_g, n_i) FP32
    S_lst: List[torch.Tensor]
    Dinv_lst: List[torch.Tensor]
    B_lst: List[torch.Tensor]
    f: torch.Tensor              # (n_leaves, n_pts, nsrc) FP64
    multi: bool
    nbr: torch.Tensor
    bnode: torch.Tensor
    tol: float = 1e-12
    max_iters: int = 30
    history: list = field(default_factory=list)


def _leaf_nodes(dom) -> np.ndarray:
    if dom.bool_2D:
        from ._grid_creation_2D import uniform_leaf_bounds_2D
        return leaf_gauss_nodes_2D(uniform_leaf_bounds_2D(dom.root.bounds, dom.L), dom.q)
    from ._grid_creation_3D import leaf_boundary_gauss_points_3D, uniform_leaf_bounds_3D
    return leaf_boundary_gauss_points_3D(uniform_leaf_bounds_3D(dom.root.bounds, dom.L), dom.q)


def _node_pairing(dom, dev):
    cache = dom.__dict__.setdefault("_refine_cache_dense", {})
    key = str(dev)
    if key not in cache:
        nbr, bnode = node_maps(_leaf_nodes(dom), dom.boundary_points, scale=dom.root.xmax - dom.root.xmin)
        cache[key] = (torch.as_tensor(nbr.astype(np.int32), device=dev),
                      torch.as_tensor(bnode.astype(np.int32), device=dev))
    return cache[key]


def _f64_to_f32(src: torch.Tensor, dst: torch.Tensor) -> None:
    nat.check(nat.lib().hps_convert(nat.HPS_F64, nat.HPS_F32, src.numel(), src.data_ptr(), dst.data_ptr(),
                                    nat.stream_ptr()), "hps_convert")


def _f32_to_f64(src: torch.Tensor, dst: torch.Tensor) -> None:
    nat.check(nat.lib().hps_convert(nat.HPS_F32, nat.HPS_F64, src.numel(), src.data_ptr(), dst.data_ptr(),
                                    nat.stream_ptr()), "hps_convert")


def _refine_leaf_operators(Y, Aii_inv, Aint, P64, Q64, Q_int, n_cb):
    """One refinement step of the FP32 leaf operators against FP64 residuals:
    R = -(A_ie P + A_ii Y0) (FP64), Y_int = Y0 + inv(A_ii) R,
    T = Q [P ; Y0] (FP64) + Q_int inv(A_ii) R.  Returns the refined T (FP32)."""
    nl, _, ng = Y.shape
    n_i = Aint.shape[1]
    dev = Y.device
    Y0 = Y[:, n_cb:, :]
    Y0_64 = torch.empty((nl, n_i, ng), dtype=torch.float64, device=dev)
    _f32_to_f64(Y0.contiguous(), Y0_64)
    R = torch.empty((nl, n_i, ng), dtype=torch.float64, device=dev)
    nat.gemm(Aint[:, :, :n_cb], P64, R, alpha=-1.0)
    nat.gemm(Aint[:, :, n_cb:], Y0_64, R, alpha=-1.0, beta=1.0, Cmat=R)
    r32 = torch.empty((nl, n_i, ng), dtype=torch.float32, device=dev)
    _f64_to_f32(R, r32)
    del R
    dY = torch.empty_like(r32)
    nat.gemm(Aii_inv, r32, dY)
    nat.gemm(Aii_inv, r32, Y0, 1.0, 1.0, Cmat=Y0)       # Y_int += dY (in place)
    QbP = torch.empty((ng, ng), dtype=torch.float64, device=dev)
    nat.gemm(Q64[:, :n_cb], P64, QbP)
    T64 = torch.empty((nl, ng, ng), dtype=torch.float64, device=dev)
    nat.gemm(Q64[:, n_cb:], Y0_64, T64, 1.0, 1.0, Cmat=QbP)
    T = torch.empty((nl, ng, ng), dtype=torch.float32, device=dev)
    _f64_to_f32(T64, T)
    nat.gemm(Q_int, dY, T, 1.0, 1.0, Cmat=T)
    return T


def build_mixed_dense(pde_problem, return_top_T=False, device=None, tol: float = 1e-12, max_iters: int = 30,
                      leaf_refine: bool = True, top_fp64_levels: int = 0):
    """FP32 build of the HPS operators plus the FP64 interior rows A_int."""
    dom = pde_problem.domain
    if pde_problem.use_ItI or not dom.bool_uniform:
        raise NotImplementedError("this mixed-precision path serves uniform DtN trees")
    if pde_problem.source is None:
        raise ValueError("mixed precision needs the source at build time")
    L = nat.lib()
    dev = st._device(device)
    dim = 2 if dom.bool_2D else 3
    P_np, Q_np = pde_problem.P, pde_problem.Q
    n_cb, ng = P_np.shape
    n_pts = Q_np.shape[1]
    n_i = n_pts - n_cb
    nl = dom.n_leaves
    upload = st._SourceUpload(pde_problem.source, nl, n_pts, torch.float64, dev)
    ops_t, coeffs, cplx = st._coefficients(pde_problem, dev)
    if cplx:
        raise NotImplementedError("mixed precision with complex coefficients is not implemented")
    Y, T, _, _, Aii = st._local_solve_dtn(pde_problem, P_np, Q_np, dev, torch.float32, keep_inverse=True,
                                          want_source=False)
    Aint = torch.empty((nl, n_i, n_pts), dtype=torch.float64, device=dev)
    nat.check(L.hps_assemble_rows(nl, n_pts, n_cb, n_i, ops_t.shape[0], ops_t.data_ptr(), coeffs.data_ptr(),
                                  Aint.data_ptr(), n_pts, n_i * n_pts, nat.stream_ptr()), "hps_assemble_rows")
    P64 = torch.as_tensor(np.ascontiguousarray(P_np), dtype=torch.float64, device=dev)
    Q64 = torch.as_tensor(np.ascontiguousarray(Q_np), dtype=torch.float64, device=dev)
    Q_int = torch.as_tensor(np.ascontiguousarray(Q_np[:, n_cb:]), dtype=torch.float32, device=dev)
    if leaf_refine:
        T = _refine_leaf_operators(Y, Aii, Aint, P64, Q64, Q_int, n_cb)
    maps_ext = _maps_for_ext(dim)
    ext_per_child = 2 if dim == 2 else 4           # a child boundary of nb points -> parent exterior nb*k
    n_levels = max(dom.L, 1) if dim == 2 else dom.L
    S_lst, Dinv_lst, B_lst, infos = [], [], [], []
    Tc = T
    for lvl in range(n_levels):
        if lvl == n_levels - top_fp64_levels:
            Tc = Tc.double()
        maps = maps_ext(Tc.shape[1] * ext_per_child)
        need_T = lvl < n_levels - 1 or return_top_T
        S, _, Tc, _, Dinv, _, B = st.merge_level_dtn(Tc, None, maps, keep_D_inv=True, keep_B=True, need_T=need_T,
                                                     infos=infos)
        S_lst.append(S.float())
        Dinv_lst.append(Dinv.float())
        B_lst.append(B.float())
    del T
    st.raise_on_sync_timeout(infos)
    f, multi = upload.result()
    nbr, bnode = _node_pairing(dom, dev)
    state = DenseMixedState(
        mixed=True, dense=True, dim=dim, n_leaves=nl, n_pts=n_pts, n_cb=n_cb, Aint=Aint, P64=P64, Q64=Q64,
        Y_int=Y[:, n_cb:, :], Aii_inv=Aii.float(), Q_int=Q_int, S_lst=S_lst, Dinv_lst=Dinv_lst, B_lst=B_lst, f=f,
        multi=multi, nbr=nbr, bnode=bnode, tol=tol, max_iters=max_iters)
    pde_problem._state = state
    pde_problem._precision = "mixed"
    pde_problem.Y = Y
    pde_problem.S_lst = S_lst
    pde_problem.D_inv_lst = Dinv_lst
    pde_problem.g_tilde_lst = []
    if return_top_T:
        return Tc[0]
    return None


def _residual(state: DenseMixedState, u_int, g, ub, r64, r32, flux):
    """FP64 residual at (u_int, g): r64 = f_int - A_int [P g ; u_int],
    flux = Q [P g ; u_int]; r32 = r64 rounded."""
    n_cb = state.n_cb
    nat.gemm(state.P64, g, ub)
    nat.gemm(state.Aint[:, :, :n_cb], ub, r64, alpha=-1.0, beta=1.0, Cmat=state.f[:, n_cb:, :])
    nat.gemm(state.Aint[:, :, n_cb:], u_int, r64, alpha=-1.0, beta=1.0, Cmat=r64)
    nat.gemm(state.Q64[:, :n_cb], ub, flux)
    nat.gemm(state.Q64[:, n_cb:], u_int, flux, 1.0, 1.0, Cmat=flux)
    _f64_to_f32(r64, r32)


def correction(state: DenseMixedState, r32, hcorr, rb32):
    """dx = M r with the FP32 operators: returns (du_int, dg) in FP32."""
    maps_ext = _maps_for_ext(state.dim)
    v = torch.empty_like(r32)
    nat.gemm(state.Aii_inv, r32, v)
    h = torch.empty_like(hcorr)
    nat.gemm(state.Q_int, v, h, 1.0, 1.0, Cmat=hcorr)
    g_t_lst = []
    hc = h
    for Dinv, B in zip(state.Dinv_lst, state.B_lst):
        g_t, hc = st.up_level(hc, Dinv, B, maps_ext(B.shape[1]))
        g_t_lst.append(g_t)
    gch = rb32.unsqueeze(0)
    for lvl in range(len(state.S_lst) - 1, -1, -1):
        S = state.S_lst[lvl]
        gch = st.down_level(S, g_t_lst[lvl], gch, maps_ext(S.shape[2]))
    nat.gemm(state.Y_int, gch, v, 1.0, 1.0, Cmat=v)   # du_int = Y_int dg + v
    return v, gch


def solve_mixed_dense(pde_problem, boundary_data, source=None, host_device="cpu", tol=None, max_iters=None):
    state: DenseMixedState = pde_problem._state
    if source is not None:
        raise ValueError("the mixed-precision solver takes the source at build time")
    L = nat.lib()
    dev = state.Aii_inv.device
    tol = state.tol if tol is None else tol
    max_iters = state.max_iters if max_iters is None else max_iters
    ns = state.f.shape[-1]
    g_given = boundary_data if isinstance(boundary_data, torch.Tensor) else torch.as_tensor(np.asarray(boundary_data))
    g_given = g_given.to(device=dev, dtype=torch.float64)
    if g_given.dim() == 1:
        g_given = g_given.unsqueeze(-1)
    if g_given.shape[-1] != ns:
        if g_given.shape[-1] == 1:
            g_given = g_given.expand(-1, ns)
        else:
            raise ValueError("boundary data and source have different numbers of right-hand sides")
    g_given = g_given.contiguous()
    nl, n_pts, n_cb = state.n_leaves, state.n_pts, state.n_cb
    n_i, ng = n_pts - n_cb, state.P64.shape[1]
    u_int = torch.zeros((nl, n_i, ns), dtype=torch.float64, device=dev)
    g = torch.zeros((nl, ng, ns), dtype=torch.float64, device=dev)
    ub = torch.empty((nl, n_cb, ns), dtype=torch.float64, device=dev)
    r32 = torch.empty((nl, n_i, ns), dtype=torch.float32, device=dev)
    r64 = torch.empty((nl, n_i, ns), dtype=torch.float64, device=dev)
    flux = torch.zeros((nl, ng, ns), dtype=torch.float64, device=dev)
    hcorr = torch.empty((nl, ng, ns), dtype=torch.float32, device=dev)
    rb32 = torch.empty((g_given.shape[0], ns), dtype=torch.float32, device=dev)
    sp = nat.stream_ptr()
    nat.check(L.hps_interior_f32(nl, n_pts, n_cb, ns, state.f.data_ptr(), r32.data_ptr(), sp), "hps_interior_f32")
    maxima = torch.empty(2, dtype=torch.float64, device=dev)
    state.history = []
    for it in range(max_iters):
        nat.check(L.hps_flux_combine(nl * ng, ns, state.nbr.data_ptr(), flux.data_ptr(), hcorr.data_ptr(),
                                     g_given.shape[0], state.bnode.data_ptr(), g_given.data_ptr(), g.data_ptr(),
                                     rb32.data_ptr(), sp), "hps_flux_combine")
        du, dg = correction(state, r32, hcorr, rb32)
        nat.check(L.hps_accumulate(dg.numel(), dg.data_ptr(), g.data_ptr(), sp), "hps_accumulate")
        step, size = nat.accumulate_max(du, u_int, maxima)
        state.history.append(step / max(size, 1e-300))
        if converged(state.history, tol):
            break
        _residual(state, u_int, g, ub, r64, r32, flux)
    else:
        raise_not_converged(state.history, tol, max_iters, "mixed-precision 3D solve")
    nat.raise_on_tc_timeout("mixed-precision 3D solve")
    u = torch.empty((nl, n_pts, ns), dtype=torch.float64, device=dev)
    nat.gemm(state.P64, g, u[:, :n_cb, :])
    u[:, n_cb:, :].copy_(u_int)
    if not state.multi:
        u = u[..., 0]
    return st._to_host(u, host_device)

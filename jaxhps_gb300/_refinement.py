"""Mixed-precision build and iteratively refined solve (uniform 2D DtN).

Build (FP32): leaf inverses inv(A_ii), the interior rows of Y, and for every
merge level S, inv(D) and B — the operators of a complete FP32 HPS direct
solver, used here as an approximate inverse M of the discrete system J.

Solve: x = (interior values u_int of every leaf, Gauss boundary values g of
every leaf) in FP64, starting from zero, iterating

    r  = b - J x                 FP64 residual after the first correction
                                 (hps_residual_2d_df), then kept current by
                                 r -= J dx in double-float with r held as
                                 an FP32 pair (hps_residual_update_2d_df);
                                 interface terms by hps_flux_combine
    dx = M r                     FP32: leaf inverse, up pass (hps_up_level),
                                 down pass (hps_down_level)
    x += dx                      FP64 (hps_accumulate)

until the remaining error is at most tol * max|u| (``converged``: the last
correction, or the contraction-rate estimate of what is left).  J is the
system the reference's FP64 direct solver solves exactly: leaf collocation
rows (local_solve/_uniform_2D_DtN.py:228-273), continuity of the outward normal derivative across interfaces
(the merge equations, merge/_schur_complement.py:182-237) and the Dirichlet
data on the domain boundary.  The fixed point is therefore the FP64 discrete
solution; each iteration contracts the error by roughly the FP32 solver's
relative accuracy.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List

import numpy as np
import torch

from . import _native as nat
from . import _phases as phases
from . import _stages as st
from ._grid_creation_2D import rearrange_indices_ext_int, uniform_leaf_bounds_2D
from ._index_maps import quad_merge_maps_dtn
from ._pdeproblem import COEFF_NAMES_2D
from ._quadrature import (
    affine_transform,
    barycentric_lagrange_interpolation_matrix_1D,
    chebyshev_points,
    differentiation_matrix_1D,
    gauss_points,
)

OP_KIND_2D = {name: i for i, name in enumerate(COEFF_NAMES_2D)}


def leaf_gauss_nodes_2D(bounds: np.ndarray, q: int) -> np.ndarray:
    """(n_leaves, 4q, 2) Gauss nodes of every leaf boundary in leaf order:
    S (x up), E (y up), N (x down), W (y down)."""
    gp = gauss_points(q)
    xmin, xmax, ymin, ymax = (bounds[:, i:i + 1] for i in range(4))
    xs = 0.5 * (xmax - xmin) * gp[None] + 0.5 * (xmin + xmax)
    ys = 0.5 * (ymax - ymin) * gp[None] + 0.5 * (ymin + ymax)
    S = np.stack([xs, np.broadcast_to(ymin, xs.shape)], -1)
    E = np.stack([np.broadcast_to(xmax, ys.shape), ys], -1)
    N = np.stack([xs[:, ::-1], np.broadcast_to(ymax, xs.shape)], -1)
    W = np.stack([np.broadcast_to(xmin, ys.shape), ys[:, ::-1]], -1)
    return np.concatenate([S, E, N, W], axis=1)


def node_maps(leaf_nodes: np.ndarray, boundary_points: np.ndarray, scale: float):
    """Pairs every leaf boundary Gauss node with the coinciding node of the
    neighbouring leaf (-1 on the domain boundary), and maps every root
    boundary point to its leaf node.  Nodes are matched by coordinates."""
    n_leaves, nb, d = leaf_nodes.shape
    flat = leaf_nodes.reshape(-1, d)
    key = np.round(flat / scale * 1e10).astype(np.int64)
    uniq, inv, counts = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    inv = inv.reshape(-1)
    order = np.argsort(inv, kind="stable")
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    nbr = np.full(flat.shape[0], -1, dtype=np.int64)
    if counts.max() > 2:
        raise ValueError("a Gauss node is shared by more than two leaves (non-conforming mesh)")
    two = np.nonzero(counts == 2)[0]
    a = order[starts[two]]
    b = order[starts[two] + 1]
    nbr[a] = b
    nbr[b] = a
    bkey = np.round(boundary_points / scale * 1e10).astype(np.int64)
    lookup = {tuple(k): i for i, k in enumerate(uniq)}
    bnode = np.empty(len(bkey), dtype=np.int64)
    for j, k in enumerate(bkey):
        u = lookup.get(tuple(k))
        if u is None or counts[u] != 1:
            raise ValueError("root boundary point does not match a single leaf boundary node")
        bnode[j] = order[starts[u]]
    return nbr, bnode


@dataclass
class MixedState:
    mixed: bool
    n_leaves: int
    p: int
    q: int
    Y_int: torch.Tensor          # (n_leaves, n_i, 4q) FP32 view
    Aii_inv: torch.Tensor        # (n_leaves, n_i, n_i) FP32
    Q_int: torch.Tensor          # (4q, n_i) FP32
    S_lst: List[torch.Tensor]
    Dinv_lst: List[torch.Tensor]
    B_lst: List[torch.Tensor]
    coeffs: torch.Tensor         # (n_ops, n_leaves, p^2) FP64
    op_kind: List[int]
    f: torch.Tensor              # (n_leaves, p^2, nsrc) FP64
    multi: bool
    consts: dict
    nbr: torch.Tensor
    bnode: torch.Tensor
    tol: float = 1e-12
    max_iters: int = 30
    history: list = field(default_factory=list)


def _domain_constants(dom, dev):
    """Residual-kernel constants and the leaf node pairing of a uniform 2D
    domain, computed once per (domain, device) and cached on the Domain."""
    cache = dom.__dict__.setdefault("_refine_cache", {})
    key = str(dev)
    if key in cache:
        return cache[key]
    p, q, n_leaves = dom.p, dom.q, dom.n_leaves
    half = (dom.root.xmax - dom.root.xmin) / (2 ** (dom.L + 1))
    cheb = chebyshev_points(p)
    D1 = differentiation_matrix_1D(cheb)
    bounds = uniform_leaf_bounds_2D(dom.root.bounds, dom.L)
    nodes = leaf_gauss_nodes_2D(bounds, q)
    nbr, bnode = node_maps(nodes, dom.boundary_points, scale=dom.root.xmax - dom.root.xmin)
    consts = {
        "inv_half": torch.full((n_leaves,), 1.0 / half, dtype=torch.float64, device=dev),
        "D1": torch.as_tensor(D1, device=dev),
        "D2": torch.as_tensor(D1 @ D1, device=dev),
        "Pside": torch.as_tensor(barycentric_lagrange_interpolation_matrix_1D(gauss_points(q), cheb), device=dev),
        "Qside": torch.as_tensor(barycentric_lagrange_interpolation_matrix_1D(cheb, gauss_points(q)), device=dev),
        "perm": torch.as_tensor(rearrange_indices_ext_int(p).astype(np.int32), device=dev),
        "nbr": torch.as_tensor(nbr.astype(np.int32), device=dev),
        "bnode": torch.as_tensor(bnode.astype(np.int32), device=dev),
    }
    cache[key] = consts
    return consts


def _refine_leaf_operators(dom, coeffs, op_kind, consts, Y, Aii_inv, Q_int):
    """One refinement step of the FP32 leaf solution operators.

    Y_int solves A_ii Y_int = W, W = -A_ie P.  With the FP32 solution Y0,
    R = W - A_ii Y0 and T0 = Q [P ; Y0] are evaluated in double-float
    arithmetic (the residual update applied to the 4q Gauss-data columns),
    then Y_int = Y0 + inv(A_ii) R and T = T0 + Q_int inv(A_ii) R in FP32.
    FP32 evaluation of W and Q Y cancels terms ~1e8 times larger than the
    DtN map's smallest eigenvalues (the near-constant modes); this step
    restores those modes to FP32 rounding level.  Returns the refined T."""
    n_leaves, n_pts, nq = Y.shape
    p, q = dom.p, dom.q
    n_cb = 4 * (p - 1)
    dev = Y.device
    Y0 = Y[:, n_cb:, :].contiguous()
    dg = torch.eye(nq, dtype=torch.float32, device=dev).expand(n_leaves, nq, nq).contiguous()
    pairs = bool(nat.lib().hps_residual_df_supported(p, q))
    r64 = None if pairs else torch.zeros(Y0.shape, dtype=torch.float64, device=dev)
    r_lo = torch.zeros(Y0.shape, dtype=torch.float32, device=dev) if pairs else None
    r32 = torch.zeros(Y0.shape, dtype=torch.float32, device=dev)
    T0 = torch.zeros((n_leaves, nq, nq), dtype=torch.float64, device=dev)
    a = nat.Residual2DArgs(
        n_leaves=n_leaves, p=p, q=q, nsrc=nq, n_ops=len(op_kind), coeffs=coeffs.data_ptr(),
        inv_half=consts["inv_half"].data_ptr(), D1=consts["D1"].data_ptr(), D2=consts["D2"].data_ptr(),
        Pside=consts["Pside"].data_ptr(), Qside=consts["Qside"].data_ptr(), perm=consts["perm"].data_ptr(),
        u_int=None, g=None, f=None, r_int=r32.data_ptr(), r_int64=nat.ptr(r64), flux=T0.data_ptr(), u_full=None)
    for i, k in enumerate(op_kind):
        a.op_kind[i] = k
    if pairs:
        prep = _df_prepare(a)
        nat.check(nat.lib().hps_residual_update_2d_df(C.byref(a), prep.data_ptr(), Y0.data_ptr(), dg.data_ptr(),
                                                      r_lo.data_ptr(), nat.stream_ptr()), "hps_residual_update_2d_df")
    else:
        nat.check(nat.lib().hps_residual_update_2d(C.byref(a), Y0.data_ptr(), dg.data_ptr(), nat.stream_ptr()),
                  "hps_residual_update_2d")
    dY = torch.empty_like(r32)
    nat.gemm(Aii_inv, r32, dY)                      # dY = inv(A_ii) R
    Y_int = Y[:, n_cb:, :]
    nat.gemm(Aii_inv, r32, Y_int, 1.0, 1.0, Cmat=Y0)  # Y_int = Y0 + dY
    T = torch.empty((n_leaves, nq, nq), dtype=torch.float32, device=dev)
    nat.check(nat.lib().hps_convert(nat.HPS_F64, nat.HPS_F32, T0.numel(), T0.data_ptr(), T.data_ptr(),
                                    nat.stream_ptr()), "hps_convert")
    nat.gemm(Q_int, dY, T, 1.0, 1.0, Cmat=T)        # T = T0 + Q_int dY
    return T


def build_mixed(pde_problem, return_top_T=False, device=None, tol: float = 1e-12, max_iters: int = 30,
                leaf_dtype=torch.float32, merge_dtype=torch.float32, top_fp64_levels: int = 0,
                leaf_refine: bool = True):
    """FP32 build of the solver operators (see module docstring).  leaf_dtype /
    merge_dtype / top_fp64_levels select the arithmetic of the leaf stage, of
    the merges and of the top merge levels; the stored operators are FP32."""
    dom = pde_problem.domain
    if pde_problem.use_ItI or not dom.bool_2D or not dom.bool_uniform:
        raise NotImplementedError("mixed precision is implemented for uniform 2D DtN problems")
    if pde_problem.source is None:
        raise ValueError("mixed precision needs the source at build time")
    dev = st._device(device)
    p, q, n_leaves = dom.p, dom.q, dom.n_leaves
    n_cb = 4 * (p - 1)
    # coefficients first: the source copy below shares the host-to-device copy
    # engine, and the leaf stage needs the coefficients, not the source
    ops_t, coeffs, cplx = st._coefficients(pde_problem, dev)
    if cplx:
        raise NotImplementedError("mixed precision with complex coefficients is not implemented")
    names = [n for n in COEFF_NAMES_2D if getattr(pde_problem, f"{n}_coefficients") is not None]
    # the interior columns of Q, on the device before the source upload starts
    Q32 = st._device_copy(pde_problem, "Q_int", lambda: np.ascontiguousarray(pde_problem.Q[:, n_cb:]),
                          torch.float32, dev)
    upload = st._SourceUpload(pde_problem.source, n_leaves, p * p, torch.float64, dev)
    Y, T, _, _, Aii = st._local_solve_dtn(pde_problem, pde_problem.P, pde_problem.Q, dev, leaf_dtype,
                                          keep_inverse=True, want_source=False,
                                          coefficients=(ops_t, coeffs, cplx))
    Y, Aii = Y.float(), Aii.float()
    consts = _domain_constants(dom, dev)
    if leaf_refine and leaf_dtype == torch.float32:
        T = _refine_leaf_operators(dom, coeffs, [OP_KIND_2D[n] for n in names], consts, Y, Aii, Q32)
    S_lst, Dinv_lst, B_lst, infos = [], [], [], []
    Tc = T.to(merge_dtype)
    n_levels = max(dom.L, 1)
    for lvl in range(n_levels):
        maps = quad_merge_maps_dtn(Tc.shape[1] // 4)
        if lvl == dom.L - top_fp64_levels:
            Tc = Tc.double()
        need_T = lvl < n_levels - 1 or return_top_T
        S, _, Tc, _, Dinv, _, B = st.merge_level_dtn(Tc, None, maps, keep_D_inv=True, keep_B=True, need_T=need_T,
                                                     infos=infos)
        S_lst.append(S.float())
        Dinv_lst.append(Dinv.float())
        B_lst.append(B.float())
    del T
    st.raise_on_sync_timeout(infos)

    f, multi = upload.result()

    state = MixedState(
        mixed=True, n_leaves=n_leaves, p=p, q=q, Y_int=Y[:, n_cb:, :], Aii_inv=Aii, Q_int=Q32, S_lst=S_lst,
        Dinv_lst=Dinv_lst, B_lst=B_lst, coeffs=coeffs, op_kind=[OP_KIND_2D[n] for n in names], f=f, multi=multi,
        consts=consts, nbr=consts["nbr"], bnode=consts["bnode"], tol=tol, max_iters=max_iters)
    pde_problem._state = state
    pde_problem._precision = "mixed"
    phases.mark("build")
    pde_problem.Y = Y
    pde_problem.S_lst = S_lst
    pde_problem.D_inv_lst = Dinv_lst
    pde_problem.g_tilde_lst = []
    if return_top_T:
        return Tc[0]
    return None


def converged(history, tol: float) -> bool:
    """True once the refinement's remaining error is at most tol (max norms,
    relative to the solution).  ``history`` holds max|dx_k| / max|x| of every
    correction so far.  Refinement converges linearly: with contraction rho,
    the error left after correction k is about rho / (1 - rho) * |dx_k|, so
    once two corrections give rho = |dx_k| / |dx_(k-1)| < 1/4 that estimate
    decides, which ends one correction before the next one would itself fall
    below tol.  Without a rate (first correction) or with slow contraction
    (rho >= 1/4, e.g. at the rounding floor), the last correction must be
    below tol."""
    h = history[-1]
    if h <= tol:
        return True
    if len(history) >= 2 and history[-2] > 0.0:
        rho = h / history[-2]
        if rho < 0.25 and rho / (1.0 - rho) * h <= tol:
            return True
    return False


def raise_not_converged(history, tol, max_iters, what: str) -> None:
    """Refinement ran max_iters steps without its last correction falling to
    tol times the solution (max norms): the result is not FP64-accurate."""
    last = f"{history[-1]:.2e}" if history else "none"
    raise nat.RefinementNotConverged(f"{what}: iterative refinement did not converge in {max_iters} steps "
                                     f"(last correction / solution = {last}, tolerance {tol:.1e})")


def _res_args(state: MixedState, u_int, g, r32, flux, r64=None, u_full=None, zero_source=False):
    c = state.consts
    a = nat.Residual2DArgs(
        n_leaves=state.n_leaves, p=state.p, q=state.q, nsrc=r32.shape[-1], n_ops=len(state.op_kind),
        coeffs=state.coeffs.data_ptr(), inv_half=c["inv_half"].data_ptr(), D1=c["D1"].data_ptr(),
        D2=c["D2"].data_ptr(), Pside=c["Pside"].data_ptr(), Qside=c["Qside"].data_ptr(), perm=c["perm"].data_ptr(),
        u_int=nat.ptr(u_int), g=nat.ptr(g), f=None if zero_source else state.f.data_ptr(),
        r_int=r32.data_ptr(), r_int64=nat.ptr(r64), flux=flux.data_ptr(), u_full=nat.ptr(u_full))
    for i, k in enumerate(state.op_kind):
        a.op_kind[i] = k
    return a


@phases.ranged("FP64 residual")
def _residual(state: MixedState, u_int, g, r32, flux, u_full=None, zero_source=False, r64=None, r_lo=None,
              u32=None):
    """FP64 residual of the discrete system at (u_int, g); zero_source drops f.
    With r_lo the leaf-row residual is also stored as the FP32 pair (r32, r_lo);
    u32 (FP32) then may give the interior values in place of u_int."""
    a = _res_args(state, u_int, g, r32, flux, r64=r64, u_full=u_full, zero_source=zero_source)
    if r_lo is not None:
        nat.check(nat.lib().hps_residual_2d_df(C.byref(a), nat.ptr(u32), r_lo.data_ptr(), nat.stream_ptr()),
                  "hps_residual_2d_df")
    else:
        nat.check(nat.lib().hps_residual_2d(C.byref(a), nat.stream_ptr()), "hps_residual_2d")


def _residual_update(state: MixedState, du, dg, r64, r32, flux):
    """r64 -= (A du)_int, flux += Q du_full (double-float arithmetic)."""
    a = _res_args(state, None, None, r32, flux, r64=r64)
    nat.check(nat.lib().hps_residual_update_2d(C.byref(a), du.data_ptr(), dg.data_ptr(), nat.stream_ptr()),
              "hps_residual_update_2d")


def _df_prepare(a) -> torch.Tensor:
    """The FP32-pair operator and coefficient table of the pair residual
    (hps_residual_df_prepare) for the problem described by the args ``a``."""
    L = nat.lib()
    nbytes = L.hps_residual_df_prep_size(a.n_leaves, a.p, a.q, a.n_ops)
    if nbytes == 0:
        raise ValueError(f"the pair residual does not serve p = {a.p}, q = {a.q}")
    prep = torch.empty(nbytes // 4, dtype=torch.float32, device=torch.device("cuda", torch.cuda.current_device()))
    nat.check(L.hps_residual_df_prepare(C.byref(a), prep.data_ptr(), nat.stream_ptr()), "hps_residual_df_prepare")
    return prep


@phases.ranged("pair residual update")
def _residual_update_df(state: MixedState, prep, du, dg, r_lo, r32, flux):
    """(r32, r_lo) -= (A du)_int as an FP32 pair, flux += Q du_full
    (double-float arithmetic, one grid line per thread); ``prep`` from
    _df_prepare."""
    a = _res_args(state, None, None, r32, flux)
    nat.check(nat.lib().hps_residual_update_2d_df(C.byref(a), prep.data_ptr(), du.data_ptr(), dg.data_ptr(),
                                                  r_lo.data_ptr(), nat.stream_ptr()), "hps_residual_update_2d_df")


@phases.ranged("correction (FP32 operators)")
def correction(state: MixedState, r32, hcorr, rb32):
    """dx = M r with the FP32 operators: returns (du_int, dg) in FP32."""
    v = torch.empty_like(r32)
    nat.gemm(state.Aii_inv, r32, v)
    h = torch.empty_like(hcorr)
    nat.gemm(state.Q_int, v, h, 1.0, 1.0, Cmat=hcorr)
    g_t_lst = []
    hc = h
    for lvl, (Dinv, B) in enumerate(zip(state.Dinv_lst, state.B_lst)):
        maps = quad_merge_maps_dtn(B.shape[1] // 8)
        g_t, hc = st.up_level(hc, Dinv, B, maps)
        g_t_lst.append(g_t)
    gch = rb32.unsqueeze(0)
    for lvl in range(len(state.S_lst) - 1, -1, -1):
        S = state.S_lst[lvl]
        gch = st.down_level(S, g_t_lst[lvl], gch, quad_merge_maps_dtn(S.shape[2] // 8))
    du = v  # du_int = Y_int dg + v   (in place on v)
    nat.gemm(state.Y_int, gch, du, 1.0, 1.0, Cmat=v)
    return du, gch


def solve_mixed(pde_problem, boundary_data, source=None, host_device="cpu", tol=None, max_iters=None, out=None):
    """The refined solve.  ``out``: a page-locked, contiguous FP64 CPU tensor of
    the result's shape receives the solution straight from the assembly
    kernel (written through its device mapping: no device-side result and no
    separate copy); it is returned once the stream has finished."""
    state: MixedState = pde_problem._state
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
    phases.mark("boundary_h2d")
    nl, p, q = state.n_leaves, state.p, state.q
    n_i = p * p - 4 * (p - 1)
    # the leaf-row residual between updates and the interior solution: FP32
    # pairs (r32, r_lo), (u_hi, u_lo) where the pair kernels serve (p, q), else FP64
    pairs = bool(L.hps_residual_df_supported(p, q))
    if pairs:
        u_int = None
        u_hi = torch.zeros((nl, n_i, ns), dtype=torch.float32, device=dev)
        u_lo = torch.zeros((nl, n_i, ns), dtype=torch.float32, device=dev)
    else:
        u_int = torch.zeros((nl, n_i, ns), dtype=torch.float64, device=dev)
    g = torch.zeros((nl, 4 * q, ns), dtype=torch.float64, device=dev)
    r32 = torch.empty((nl, n_i, ns), dtype=torch.float32, device=dev)
    r64 = None if pairs else torch.empty((nl, n_i, ns), dtype=torch.float64, device=dev)
    r_lo = torch.empty((nl, n_i, ns), dtype=torch.float32, device=dev) if pairs else None
    flux = torch.zeros((nl, 4 * q, ns), dtype=torch.float64, device=dev)
    prep = _df_prepare(_res_args(state, None, None, r32, flux)) if pairs else None
    hcorr = torch.empty((nl, 4 * q, ns), dtype=torch.float32, device=dev)
    rb32 = torch.empty((g_given.shape[0], ns), dtype=torch.float32, device=dev)
    sp = nat.stream_ptr()
    # residual at x = 0 is b itself
    nat.check(L.hps_interior_f32(nl, p * p, 4 * (p - 1), ns, state.f.data_ptr(), r32.data_ptr(), sp),
              "hps_interior_f32")
    maxima = torch.empty(2, dtype=torch.float64, device=dev)
    state.history = []
    for it in range(max_iters):
        nat.check(L.hps_flux_combine(nl * 4 * q, ns, state.nbr.data_ptr(), flux.data_ptr(), hcorr.data_ptr(),
                                     g_given.shape[0], state.bnode.data_ptr(), g_given.data_ptr(), g.data_ptr(),
                                     rb32.data_ptr(), sp), "hps_flux_combine")
        du, dg = correction(state, r32, hcorr, rb32)
        nat.check(L.hps_accumulate(dg.numel(), dg.data_ptr(), g.data_ptr(), sp), "hps_accumulate")
        if pairs:
            step, size = nat.accumulate_max_df(du, u_hi, u_lo, maxima)
        else:
            step, size = nat.accumulate_max(du, u_int, maxima)
        state.history.append(step / max(size, 1e-300))
        if converged(state.history, tol):
            break
        if it == 0:
            # the first correction is the size of the solution: recompute the
            # residual from scratch in FP64
            # (with pairs the interior solution is still du of the first
            # correction, exactly u_hi)
            _residual(state, u_int, g, r32, flux, r64=r64, r_lo=r_lo, u32=u_hi if pairs else None)
        elif pairs:
            _residual_update_df(state, prep, du, dg, r_lo, r32, flux)
        else:
            _residual_update(state, du, dg, r64, r32, flux)
    else:
        raise_not_converged(state.history, tol, max_iters, "mixed-precision DtN solve")
    nat.raise_on_tc_timeout("mixed-precision DtN solve")
    shape = (nl, p * p, ns) if state.multi else (nl, p * p)
    dst = None
    if (out is not None and tuple(out.shape) == shape and out.dtype == torch.float64 and out.is_contiguous()):
        dst = nat.mapped_pointer(out)
    def assemble(target):
        if pairs:
            nat.check(L.hps_assemble_u_2d_df(nl, p, q, ns, state.consts["Pside"].data_ptr(), u_hi.data_ptr(),
                                             u_lo.data_ptr(), g.data_ptr(), target, sp), "hps_assemble_u_2d_df")
        else:
            nat.check(L.hps_assemble_u_2d(nl, p, q, ns, state.consts["Pside"].data_ptr(), u_int.data_ptr(),
                                          g.data_ptr(), target, sp), "hps_assemble_u_2d")

    if dst is not None:
        phases.mark("refine")
        assemble(dst)
        torch.cuda.current_stream(dev).synchronize()
        return out
    u = torch.empty((nl, p * p, ns), dtype=torch.float64, device=dev)
    assemble(u.data_ptr())
    if not state.multi:
        u = u[..., 0]
    phases.mark("refine")
    return st._to_host(u, host_device)

"""Build once without a source, solve for many sources (uniform 2D, DtN and ItI).

Mirrors _build_solver.py:261-331 (_nosource_build_solver), the no-source
leaf stages (local_solve/_nosource_uniform_2D_DtN.py:76-116,
_nosource_uniform_2D_ItI.py:80-139), the no-source merges that keep D^-1 and
B D^-1 (merge/_nosource_uniform_2D_ItI.py:19-131 and the DtN analogue), the
up passes (up_pass/_uniform_2D_DtN.py:8-173, up_pass/_uniform_2D_ItI.py
:8-214) and _solve.py's _up_then_down_pass.

Stored on the problem: ``Y``, ``Phi`` (DtN: inv(A_ii), which maps the
interior source to the interior particular solution; ItI: the source columns
of inv(B)), ``S_lst``, ``D_inv_lst`` and ``BD_inv_lst``.  The up pass works
on an internal layout (rows of B D^-1 in the merged exterior's final,
rolled order; ItI interface unknowns in the order of S's rows), kept as
``_D_inv_int`` / ``_BD_inv_int``; ``D_inv_lst`` and ``BD_inv_lst`` present
them in the reference's layout (merge/_nosource_uniform_2D_DtN.py:238-248,
merge/_nosource_uniform_2D_ItI.py: B D^-1 before the roll of the merged
exterior, ItI interface unknowns in the h_int order b5, d8, b6, d7, a5, c6,
c7, a8), converted when an element is read.
"""

from __future__ import annotations

from collections.abc import Sequence

import numpy as np
import torch

from . import _native as nat
from . import _stages as st
from ._index_maps import quad_merge_maps_dtn, quad_merge_maps_iti


def nosource_local_solve_stage_uniform_2D_DtN(pde_problem, device=None, host_device=None, dtype=torch.float64):
    """(Y, T, Phi) with Phi = inv(A_ii) per leaf."""
    Y, T, _, _, Aii = st._local_solve_dtn(pde_problem, pde_problem.P, pde_problem.Q, device, dtype, True,
                                          want_source=False)
    return Y, T, Aii


def nosource_local_solve_stage_uniform_2D_ItI(pde_problem, device=None, host_device=None,
                                              dtype=torch.complex128):
    """(Y, T, Phi) with Phi = inv(B)[:, n_cb:] per leaf."""
    src = pde_problem.source
    pde_problem.source = None
    try:
        Y, T, _, _, Binv = st.local_solve_stage_uniform_2D_ItI(pde_problem, device=device, dtype=dtype,
                                                               keep_inverse=True)
    finally:
        pde_problem.source = src
    n_cb = pde_problem.P.shape[0]
    return Y, T, Binv[:, :, n_cb:]


def _iti_order(nc: int) -> np.ndarray:
    """Position in the reference's h_int order of each interface unknown in
    S's row order (the row permutation of merge/_uniform_2D_ItI.py:360-373)."""
    return np.concatenate([np.arange(0, nc), np.arange(4 * nc, 5 * nc), np.arange(5 * nc, 6 * nc),
                           np.arange(2 * nc, 3 * nc), np.arange(3 * nc, 4 * nc), np.arange(6 * nc, 7 * nc),
                           np.arange(7 * nc, 8 * nc), np.arange(nc, 2 * nc)])


def public_D_inv(Dinv: torch.Tensor, iti: bool) -> torch.Tensor:
    """D^-1 of one level in the reference's layout."""
    if not iti:
        return Dinv
    inv = torch.as_tensor(np.argsort(_iti_order(Dinv.shape[-1] // 8)), device=Dinv.device)
    return Dinv.index_select(-2, inv).index_select(-1, inv)


def public_BD_inv(BDinv: torch.Tensor, iti: bool) -> torch.Tensor:
    """B D^-1 of one level in the reference's layout: rows before the roll of
    the merged exterior by -nc, ItI columns in the h_int order."""
    nc = BDinv.shape[-2] // 8
    out = torch.roll(BDinv, nc, dims=-2)
    if iti:
        inv = torch.as_tensor(np.argsort(_iti_order(BDinv.shape[-1] // 8)), device=BDinv.device)
        out = out.index_select(-1, inv)
    return out


class LayoutList(Sequence):
    """A read-only list whose items are converted from an internal list when
    they are read (the reference's layout of D^-1 / B D^-1)."""

    def __init__(self, items, convert):
        self._items, self._convert = items, convert

    def __len__(self):
        return len(self._items)

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self._convert(x) for x in self._items[i]]
        return self._convert(self._items[i])


def store_operators(pde_problem, Dinv_lst, BDinv_lst, iti: bool) -> None:
    """Internal lists for the up pass, reference-layout views as the public attributes."""
    pde_problem._D_inv_int, pde_problem._BD_inv_int = Dinv_lst, BDinv_lst
    pde_problem.D_inv_lst = LayoutList(Dinv_lst, lambda t: public_D_inv(t, iti))
    pde_problem.BD_inv_lst = LayoutList(BDinv_lst, lambda t: public_BD_inv(t, iti))


def _nosource_merge(T_arr, l: int, iti: bool, device=None, return_T: bool = False):
    dev = st._device(device)
    T = T_arr.to(dev).contiguous()
    S_lst, Dinv_lst, BDinv_lst, infos = [], [], [], []
    n_levels = max(int(l), 1)
    for lvl in range(n_levels):
        nc = T.shape[1] // 4
        maps = quad_merge_maps_iti(nc) if iti else quad_merge_maps_dtn(nc)
        need_T = lvl < n_levels - 1 or return_T
        S, _, T, _, Dinv, BDinv = st.merge_level_dtn(T, None, maps, keep_D_inv=True, keep_BD_inv=True, iti=iti,
                                                     need_T=need_T, infos=infos)
        S_lst.append(S)
        Dinv_lst.append(Dinv)
        BDinv_lst.append(BDinv)
    st.raise_on_sync_timeout(infos)
    out = (S_lst, Dinv_lst, BDinv_lst)
    if return_T:
        out = out + (T[0],)
    return out


def nosource_merge_stage_uniform_2D_DtN(T_arr, l: int, device=None, host_device=None, return_T: bool = False):
    """(S_lst, D_inv_lst, BD_inv_lst[, T_top])."""
    return _nosource_merge(T_arr, l, False, device, return_T)


def nosource_merge_stage_uniform_2D_ItI(T_arr, l: int, device=None, host_device=None, return_T: bool = False):
    """(S_lst, D_inv_lst, BD_inv_lst[, T_top]) (merge/_nosource_uniform_2D_ItI.py:19-131)."""
    return _nosource_merge(T_arr, l, True, device, return_T)


def nosource_build_solver(pde_problem, return_top_T: bool = False, device=None, dtype=torch.float64):
    dom = pde_problem.domain
    if not dom.bool_2D or not dom.bool_uniform:
        raise ValueError("Build stage for problems without source terms is only implemented for 2D uniform problems.")
    if pde_problem.use_ItI:
        Y, T, Phi = nosource_local_solve_stage_uniform_2D_ItI(pde_problem, device=device,
                                                              dtype=st.REAL_TO_COMPLEX.get(dtype, dtype))
    else:
        Y, T, Phi = nosource_local_solve_stage_uniform_2D_DtN(pde_problem, device=device, dtype=dtype)
    pde_problem.Y, pde_problem.Phi, pde_problem.v = Y, Phi, None
    out = _nosource_merge(T, dom.L, pde_problem.use_ItI, device, return_top_T)
    pde_problem.S_lst = out[0]
    store_operators(pde_problem, out[1], out[2], pde_problem.use_ItI)
    pde_problem.g_tilde_lst = []
    pde_problem._precision = "nosource"
    if return_top_T:
        return out[3]
    return None


def _up_pass(source, pde_problem, iti: bool, device=None, return_h_last: bool = False):
    if getattr(pde_problem, "Phi", None) is None or not getattr(pde_problem, "_D_inv_int", None):
        raise ValueError("solve(..., source=...) needs a solver built without a source (build_solver on a "
                         "PDEProblem whose source is None)")
    Phi = pde_problem.Phi
    dev, dtype = Phi.device, Phi.dtype
    f, multi = st._src3(source, Phi.shape[0], pde_problem.Y.shape[1], dtype, dev)
    n_cb = pde_problem.P.shape[0]
    nl, n_pts, ns = f.shape
    if iti:
        v = torch.empty((nl, n_pts, ns), dtype=dtype, device=dev)
        nat.gemm(Phi, f[:, n_cb:, :], v)
        Q = st._as_tensor(pde_problem.QH, dtype, dev)
    else:
        v = torch.zeros((nl, n_pts, ns), dtype=dtype, device=dev)
        nat.gemm(Phi, f[:, n_cb:, :], v[:, n_cb:, :])
        Q = st._as_tensor(pde_problem.Q, dtype, dev)
    h = torch.empty((nl, Q.shape[0], ns), dtype=dtype, device=dev)
    nat.gemm(Q, v, h)
    g_lst = []
    for Dinv, BDinv in zip(pde_problem._D_inv_int, pde_problem._BD_inv_int):
        nc = BDinv.shape[1] // 8
        maps = quad_merge_maps_iti(nc) if iti else quad_merge_maps_dtn(nc)
        g_t, h = st.up_level(h, Dinv, BDinv, maps, b_is_bd_inv=True, iti=iti)
        g_lst.append(g_t if multi else g_t[..., 0])
    if not multi:
        v = v[..., 0]
    out = (v, g_lst)
    if return_h_last:
        out = out + ((h[0] if multi else h[0, :, 0]),)
    return out


def up_pass_uniform_2D_DtN(source, pde_problem, device=None, host_device=None, return_h_last: bool = False):
    """(v, g_tilde_lst[, h_last]) for a new source (up_pass/_uniform_2D_DtN.py:8-173)."""
    return _up_pass(source, pde_problem, False, device, return_h_last)


def up_pass_uniform_2D_ItI(source, pde_problem, device=None, host_device=None, return_h_last: bool = False):
    """(v, g_tilde_lst[, h_last]) for a new source (up_pass/_uniform_2D_ItI.py:8-214)."""
    return _up_pass(source, pde_problem, True, device, return_h_last)


def up_then_down_pass(pde_problem, boundary_data, source, device=None, host_device="cpu"):
    """_solve.py _up_then_down_pass: up pass for ``source``, then the down pass."""
    if pde_problem.use_ItI:
        from . import _iti
        v, g_lst = up_pass_uniform_2D_ItI(source, pde_problem, device)
        return _iti.down_pass_uniform_2D_ItI(boundary_data, pde_problem.S_lst, g_lst, pde_problem.Y, v,
                                             device=device, host_device=host_device)
    v, g_lst = up_pass_uniform_2D_DtN(source, pde_problem, device)
    return st.down_pass_uniform_2D_DtN(boundary_data, pde_problem.S_lst, g_lst, pde_problem.Y, v, device=device,
                                       host_device=host_device)

"""ItI merge stage and down pass for uniform 2D quadtrees (GPU), mirroring
src/jaxhps/merge/_uniform_2D_ItI.py:19-179 and
src/jaxhps/down_pass/_uniform_2D_ItI.py:8-118.

The merge runs hps_merge_level_iti once per level; the down pass reuses
hps_down_level with the ItI index maps (the reference's per-side unknowns
and flips, down_pass/_uniform_2D_ItI.py:121-192)."""

from __future__ import annotations

import numpy as np
import torch

from . import _stages as st
from ._index_maps import quad_merge_maps_iti


def merge_stage_uniform_2D_ItI(T_arr, h_arr, l: int, device=None, host_device=None, subtree_recomp: bool = False,
                               return_T: bool = False, return_h: bool = False):
    """Returns (S_lst, g_tilde_lst[, T_top][, h_top]) like the reference."""
    dev = st._device(device)
    T = T_arr if isinstance(T_arr, torch.Tensor) else st._as_tensor(T_arr, torch.complex128, dev)
    T = T.to(dev).contiguous()
    if not T.is_complex():
        T = T.to(torch.complex128)
    if T.dim() == 4:
        T = T.reshape(-1, T.shape[-2], T.shape[-1])
    multi = h_arr is not None and (h_arr.dim() == 3 if isinstance(h_arr, torch.Tensor) else np.ndim(h_arr) == 3)
    h = None
    if h_arr is not None:
        h = h_arr if isinstance(h_arr, torch.Tensor) else st._as_tensor(h_arr, T.dtype, dev)
        h = h.to(device=dev, dtype=T.dtype)
        if h.dim() == 2:
            h = h.unsqueeze(-1)
        h = h.reshape(T.shape[0], T.shape[1], -1).contiguous()
    S_lst, g_lst = [], []
    for _ in range(max(int(l), 1)):
        maps = quad_merge_maps_iti(T.shape[1] // 4)
        S, g_t, T, h, _, _ = st.merge_level_dtn(T, h, maps, iti=True)
        S_lst.append(S)
        g_lst.append(g_t if (g_t is None or multi) else g_t[..., 0])
    if subtree_recomp:
        return T, (h if (h is None or multi) else h[..., 0])
    out = (S_lst, g_lst)
    if return_T:
        out = out + (T[0],)
    if return_h:
        out = out + (None if h is None else (h[0] if multi else h[0, :, 0]),)
    return out


def down_pass_uniform_2D_ItI(boundary_data, S_lst, g_tilde_lst, Y_arr, v_arr, device=None, host_device=None):
    """Propagates incoming impedance data from the root to the leaves and
    returns the leaf solutions (or the leaf impedance data when Y_arr is None)."""
    return st._down_pass_generic(boundary_data, S_lst, g_tilde_lst, Y_arr, v_arr, quad_merge_maps_iti, device,
                                 host_device)

"""3D uniform DtN merge and down-pass stages (oct merges).

The leaf stage is shared with 2D (``_stages.local_solve_stage_uniform_3D_DtN``):
the leaf algebra only sees p^3 points and 6q^2 Gauss nodes.  Merges and the
down pass run the same GPU kernels as the quad tree with the oct-merge index
maps of ``_index_maps.oct_merge_maps_dtn``.
"""

from __future__ import annotations

from . import _stages as st
from ._index_maps import oct_merge_maps_dtn


def merge_stage_uniform_3D_DtN(T_arr, h_arr, l: int, device=None, host_device=None, subtree_recomp: bool = False,
                               return_T: bool = False, keep_D_inv: bool = False):
    """Level loop of DtN oct merges (reference merge/_uniform_3D_DtN.py:12-124):
    ``l`` levels for 8^l leaves.  Returns ``(S_lst, g_tilde_lst)`` (leaf-adjacent
    level first, root last with a leading batch axis of 1) and the top-level T
    when ``return_T``."""
    if int(l) < 1:
        raise ValueError("a 3D uniform tree needs at least one level (L >= 1)")
    out = st.merge_stage_generic(T_arr, h_arr, int(l), lambda nb: oct_merge_maps_dtn(nb // 6), device,
                                 subtree_recomp, return_T, keep_D_inv)
    if subtree_recomp:
        return out
    # like the reference (merge/_uniform_3D_DtN.py:116), the root entries carry no batch axis
    S_lst, g_lst = out[0], out[1]
    S_lst[-1] = S_lst[-1][0]
    if g_lst[-1] is not None:
        g_lst[-1] = g_lst[-1][0]
    return out


def down_pass_uniform_3D_DtN(boundary_data, S_lst, g_tilde_lst, Y_arr, v_arr, device=None, host_device=None):
    """Reference down_pass/_uniform_3D_DtN.py:8-113 (one level =
    _propogate_down_oct_DtN :116-246).  Boundary data is ordered like
    ``Domain.boundary_points``; returns the leaf solutions (n_leaves, p^3[, nsrc]).
    The root entries of S_lst / g_tilde_lst have no batch axis (:86-87)."""
    S_lst = list(S_lst)
    g_tilde_lst = list(g_tilde_lst)
    if S_lst[-1].dim() == 2:
        S_lst[-1] = S_lst[-1].unsqueeze(0)
        g = g_tilde_lst[-1]
        if g is not None:
            g_tilde_lst[-1] = g.unsqueeze(0)
    return st._down_pass_generic(boundary_data, S_lst, g_tilde_lst, Y_arr, v_arr, oct_merge_maps_dtn, device,
                                 host_device, ext_per_unit=24)

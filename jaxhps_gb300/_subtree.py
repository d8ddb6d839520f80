"""Subtree-recomputation API (mirror of src/jaxhps/_subtree_recomp.py:20-541).

The reference splits a large uniform 2D tree into subtrees of height
``subtree_height`` so that the operators of the lower levels never have to
leave a small device memory: it merges each subtree to its root, merges the
roots, and during the solve recomputes every subtree.  A GB300 keeps the
whole operator set of such problems in HBM, so here the three entry points
keep their signatures and results but run the ordinary build (all levels in
HBM, no recomputation); ``subtree_height`` is accepted and ignored.
"""

from __future__ import annotations

import torch

from . import _stages as st


def _check(pde_problem):
    dom = pde_problem.domain
    if not dom.bool_2D or not dom.bool_uniform:
        raise ValueError("Subtree recomputation is only supported for 2D problems with uniform quadtrees.")


def _build(pde_problem, compute_device, return_T):
    dom = pde_problem.domain
    if pde_problem.use_ItI:
        from . import _iti
        Y, T, v, h = st.local_solve_stage_uniform_2D_ItI(pde_problem, device=compute_device)
        out = _iti.merge_stage_uniform_2D_ItI(T, h, l=dom.L, device=compute_device, return_T=return_T)
    else:
        Y, T, v, h = st.local_solve_stage_uniform_2D_DtN(pde_problem, device=compute_device)
        out = st.merge_stage_uniform_2D_DtN(T, h, l=dom.L, device=compute_device, return_T=return_T)
    return Y, v, out


def _down(pde_problem, boundary_data, S_lst, g_lst, Y, v, compute_device, host_device):
    if isinstance(boundary_data, list):
        boundary_data = torch.cat([torch.as_tensor(b) for b in boundary_data])
    if pde_problem.use_ItI:
        from . import _iti
        return _iti.down_pass_uniform_2D_ItI(boundary_data, S_lst, g_lst, Y, v, device=compute_device,
                                             host_device=host_device)
    return st.down_pass_uniform_2D_DtN(boundary_data, S_lst, g_lst, Y, v, device=compute_device,
                                       host_device=host_device)


def solve_subtree(pde_problem, boundary_data, subtree_height: int = 7, compute_device=None, host_device="cpu"):
    """Builds and solves in one call without storing any solution operator
    on the problem (_subtree_recomp.py:20-163)."""
    _check(pde_problem)
    Y, v, out = _build(pde_problem, compute_device, False)
    return _down(pde_problem, boundary_data, out[0], out[1], Y, v, compute_device, host_device)


def upward_pass_subtree(pde_problem, subtree_height: int = 7, compute_device=None, host_device="cpu"):
    """Upward pass: stores ``S_lst`` and ``g_tilde_lst`` and returns the
    top-level Poincare-Steklov matrix (_subtree_recomp.py:395-456)."""
    _check(pde_problem)
    Y, v, out = _build(pde_problem, compute_device, True)
    pde_problem.S_lst, pde_problem.g_tilde_lst = out[0], out[1]
    pde_problem._subtree_leaf_ops = (Y, v)
    return st._to_host(out[2], host_device)


def downward_pass_subtree(pde_problem, boundary_data, subtree_height: int = 7, compute_device=None,
                          host_device="cpu"):
    """Downward pass after upward_pass_subtree (_subtree_recomp.py:459-541)."""
    _check(pde_problem)
    ops = getattr(pde_problem, "_subtree_leaf_ops", None)
    if ops is None:
        raise ValueError("downward_pass_subtree needs upward_pass_subtree first")
    Y, v = ops
    return _down(pde_problem, boundary_data, pde_problem.S_lst, pde_problem.g_tilde_lst, Y, v, compute_device,
                 host_device)

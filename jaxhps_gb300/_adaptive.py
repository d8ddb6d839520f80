"""Adaptive (non-uniform) DtN build and solve, 3D octrees and 2D quadtrees.

Mirrors local_solve/_adaptive_3D_DtN.py:13-175, merge/_adaptive_3D_DtN.py
:30-565 (with merge/_utils_adaptive_3D_DtN.py) and
down_pass/_adaptive_3D_DtN.py:15-394; in 2D local_solve/_adaptive_2D_DtN.py,
merge/_adaptive_2D_DtN.py (with merge/_utils_adaptive_2D_DtN.py) and
down_pass/_adaptive_2D_DtN.py.  The text below speaks of 3D; in 2D a merge
has four children with four sides, interfaces compress two fine panels of
q points onto one coarse panel (L_1f2 rows, L_2f1 columns) and the second
side of every interface runs opposite to the first.

Leaves: one batched leaf solve; every leaf's operator uses the reference
operators (half side 1) with its coefficients rescaled by h^-order, h the
leaf's half side, and its T and h by 1/h (the per-leaf Q of the reference).

Merges, level by level from the deepest: a node's eight children are first
brought into the merge's basis — on every interface where one side has four
fine panels against one coarse panel, the fine side's rows are compressed
with L_1f4 and its columns with L_4f1 (hps_panel_map) — then the children
are zero-padded to a common size and merged by the uniform GPU merge with a
per-node index map (variable face sizes, the reference's re-ordering of
:745-881).  Nodes of a level with the same signature (children's face sizes
and compression pattern) share their maps and run as one batched merge.

Down pass: the same buckets from the root down; the children's boundary data
are scattered from (g_parent, S g_parent + g~) and compressed interface
panels are expanded back with L_4f1 (down_pass/_adaptive_3D_DtN.py
_deproject_merge_interface_3D).  Leaves: u = Y g + v.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, List, Tuple

import numpy as np
import torch

from . import _native as nat
from . import _stages as st
from ._discretization_tree import get_all_leaves, get_depth, get_nodes_at_level
from ._grid_creation_3D import FACE_TRAVERSAL, get_ordered_lst_of_boundary_nodes
from ._index_maps import CODE_PAD, OCT_CHILD_BITS, OCT_INTERFACES, maps_from_code
from ._pdeproblem import COEFF_NAMES_2D, COEFF_NAMES_3D

_ORDER_3D = {"D_xx": 2, "D_xy": 2, "D_yy": 2, "D_xz": 2, "D_yz": 2, "D_zz": 2, "D_x": 1, "D_y": 1, "D_z": 1, "I": 0}
_ORDER_2D = {"D_xx": 2, "D_xy": 2, "D_yy": 2, "D_x": 1, "D_y": 1, "I": 0}


@dataclass(frozen=True)
class _Geometry:
    """What differs between quad and oct merges."""
    dim: int
    nch: int                      # children per merge
    nsides: int                   # sides (faces) per node
    fine: int                     # fine panels facing one coarse panel
    ext_order: Tuple[Tuple[int, int], ...]                 # (child, side) of the merged exterior, in order
    interfaces: Tuple[Tuple[int, int, int, int, bool], ...]  # (child0, side0, child1, side1, side1 reversed)


def _geometry_3D() -> _Geometry:
    ext = []
    for F in range(6):
        axis, side = F // 2, F % 2
        ext += [(c, F) for c in FACE_TRAVERSAL[axis] if OCT_CHILD_BITS[c][axis] == side]
    inter = []
    for i in range(12):
        c0, c1 = OCT_INTERFACES[i]
        axis = next(k for k in range(3) if OCT_CHILD_BITS[c0][k] != OCT_CHILD_BITS[c1][k])
        lo, hi = (c0, c1) if OCT_CHILD_BITS[c0][axis] == 0 else (c1, c0)
        inter.append((lo, 2 * axis + 1, hi, 2 * axis, False))
    return _Geometry(3, 8, 6, 4, tuple(ext), tuple(inter))


# 2D: children a..d = SW, SE, NE, NW, sides S, E, N, W; merged exterior
# [a_S, b_S, b_E, c_E, c_N, d_N, d_W, a_W] and interfaces 5 (a_E | b_W),
# 6 (b_N | c_S), 7 (c_W | d_E), 8 (d_S | a_N), each second side reversed
# (the orientation of the uniform quad merge, _index_maps.quad_merge_maps_dtn).
_GEOM_2D = _Geometry(2, 4, 4, 2, ((0, 0), (1, 0), (1, 1), (2, 1), (2, 2), (3, 2), (3, 3), (0, 3)),
                     ((0, 1, 1, 3, True), (1, 2, 2, 0, True), (2, 3, 3, 1, True), (3, 0, 0, 2, True)))
_GEOM_3D = _geometry_3D()


def _geom(node) -> _Geometry:
    return _GEOM_3D if hasattr(node, "zmin") else _GEOM_2D


def _face_sizes(node) -> Tuple[int, ...]:
    if hasattr(node, "zmin"):
        return (node.n_0, node.n_1, node.n_2, node.n_3, node.n_4, node.n_5)
    return (node.n_0, node.n_1, node.n_2, node.n_3)


def _projection_lst(lst_0, lst_1, fine: int = 4):
    """Which panels of two facing leaf lists are compressed (``fine`` fine
    panels -> 1 coarse), walking both lists in step
    (merge/_utils_adaptive_3D_DtN.py:11-57, merge/_utils_adaptive_2D_DtN.py)."""
    out_0, out_1 = [], []
    i0 = i1 = 0
    while i0 < len(lst_0) and i1 < len(lst_1):
        s0 = lst_0[i0].xmax - lst_0[i0].xmin
        s1 = lst_1[i1].xmax - lst_1[i1].xmin
        if s0 == s1:
            out_0.append(False)
            out_1.append(False)
            i0 += 1
            i1 += 1
        elif s0 < s1:
            out_0 += [True] * fine
            out_1.append(False)
            i0 += fine
            i1 += 1
        else:
            out_1 += [True] * fine
            out_0.append(False)
            i1 += fine
            i0 += 1
    return tuple(out_0), tuple(out_1)


def _boundary_leaf_lists(node):
    if hasattr(node, "zmin"):
        return get_ordered_lst_of_boundary_nodes(node)
    from ._discretization_tree_operations_2D import get_ordered_lst_of_boundary_nodes as lst2
    return lst2(node)


def projection_lists(node) -> Dict[Tuple[int, int], Tuple[bool, ...]]:
    """(child, side) -> panel compression flags, in the side's own order, on
    every interface of a merge (find_projection_lists_3D,
    merge/_utils_adaptive_3D_DtN.py:60-166; find_compression_lists_2D)."""
    g = _geom(node)
    leaves = [_boundary_leaf_lists(ch) for ch in node.children]
    out = {}
    for c0, s0, c1, s1, rev in g.interfaces:
        l1 = leaves[c1][s1][::-1] if rev else leaves[c1][s1]
        a, b = _projection_lst(leaves[c0][s0], l1, g.fine)
        out[(c0, s0)] = a
        out[(c1, s1)] = b[::-1] if rev else b
    return out


@dataclass
class MergePlan:
    """Everything a merge needs that depends only on its signature."""
    sizes: Tuple[Tuple[int, ...], ...]       # full face sizes per child
    red_sizes: Tuple[Tuple[int, ...], ...]   # face sizes in the merge basis
    nb: Tuple[int, ...]                      # full boundary size per child
    nbr: Tuple[int, ...]                     # reduced boundary size per child
    nbr_max: int
    n_ext: int
    n_int: int
    maps: object
    compress: List[torch.Tensor]             # per child, int32 (nbr_c, 4) tables (device)
    expand: List[torch.Tensor]               # per child, int32 (nb_c, 4) tables (device)
    any_compressed: Tuple[bool, ...]


def _build_plan(sizes, proj, q: int, dev, g: _Geometry = None) -> MergePlan:
    g = _GEOM_3D if g is None else g
    pan = q ** (g.dim - 1)          # points of one panel (q^2 on a face, q on a side)
    red_sizes = []
    compress, expand = [], []
    for c in range(g.nch):
        rs = []
        ctab, etab = [], []
        off_full = off_red = 0
        for f in range(g.nsides):
            n = sizes[c][f]
            flags = proj.get((c, f))
            if flags is None:                           # exterior side: unchanged
                for t in range(n):
                    ctab.append((0, off_full, t, 0))
                    etab.append((0, off_red, t, 0))
                rs.append(n)
            else:
                if len(flags) * pan != n:
                    raise ValueError("face panel count does not match the node's face size")
                pi = red = 0
                while pi < len(flags):
                    if flags[pi]:
                        for l in range(pan):
                            ctab.append((1, off_full + pi * pan, l, g.fine * pan))
                        for l in range(g.fine * pan):
                            etab.append((1, off_red + red, l, pan))
                        pi += g.fine
                    else:
                        for l in range(pan):
                            ctab.append((0, off_full + pi * pan, l, 0))
                            etab.append((0, off_red + red, l, 0))
                        pi += 1
                    red += pan
                rs.append(red)
            off_full += n
            off_red += rs[-1]
        red_sizes.append(tuple(rs))
        compress.append(torch.as_tensor(np.array(ctab, dtype=np.int32).reshape(-1, 4), device=dev))
        expand.append(torch.as_tensor(np.array(etab, dtype=np.int32).reshape(-1, 4), device=dev))
    nb = tuple(sum(sz) for sz in sizes)
    nbr = tuple(sum(sz) for sz in red_sizes)
    nbr_max = max(nbr)
    code = np.full((g.nch, nbr_max), CODE_PAD, dtype=np.int64)
    red_off = [np.concatenate([[0], np.cumsum(red_sizes[c])[:-1]]) for c in range(g.nch)]
    ext = 0
    for c, F in g.ext_order:
        n = red_sizes[c][F]
        code[c, red_off[c][F]:red_off[c][F] + n] = ext + np.arange(n)
        ext += n
    it = 0
    for c0, s0, c1, s1, rev in g.interfaces:
        m = red_sizes[c0][s0]
        if red_sizes[c1][s1] != m:
            raise ValueError("interface sides do not match after compression")
        idx = -(it + np.arange(m) + 1)
        code[c0, red_off[c0][s0]:red_off[c0][s0] + m] = idx
        code[c1, red_off[c1][s1]:red_off[c1][s1] + m] = idx[::-1] if rev else idx
        it += m
    maps = maps_from_code(code, n_ext=ext, n_int=it)
    anyc = tuple(any(proj.get((c, f), ()) and any(proj[(c, f)]) for f in range(g.nsides)) for c in range(g.nch))
    return MergePlan(tuple(tuple(sz) for sz in sizes), tuple(red_sizes), nb, nbr, nbr_max, ext, it, maps, compress,
                     expand, anyc)


@dataclass
class Bucket:
    nodes: list
    plan: MergePlan
    S: torch.Tensor
    g_tilde: torch.Tensor


def _leaf_coefficients(pde_problem, dev):
    """Active (ops, per-leaf rescaled coeffs, complex flag) for adaptive leaves."""
    ops_t, coeffs, cplx = st._coefficients(pde_problem, dev)
    two_d = pde_problem.domain.bool_2D
    order = _ORDER_2D if two_d else _ORDER_3D
    names = [n for n in (COEFF_NAMES_2D if two_d else COEFF_NAMES_3D)
             if getattr(pde_problem, f"{n}_coefficients") is not None]
    h = np.asarray(pde_problem.sidelens, dtype=np.float64) / 2.0
    scale = np.stack([h ** (-order[n]) for n in names])              # (n_ops, n_leaves)
    sc = torch.as_tensor(np.ascontiguousarray(scale), device=dev)
    coeffs = coeffs.clone()
    dt = nat.TORCH_TO_HPS[coeffs.dtype]
    nat.check(nat.lib().hps_scale_batched(dt, sc.numel(), coeffs.shape[-1], sc.data_ptr(), coeffs.data_ptr(),
                                          nat.stream_ptr()), "hps_scale_batched")
    return ops_t, coeffs, cplx


def local_solve_stage_adaptive_3D_DtN(pde_problem, device=None, host_device=None, dtype=torch.float64):
    """Leaf DtN maps of an adaptive octree (local_solve/_adaptive_3D_DtN.py:13-175)
    or quadtree (local_solve/_adaptive_2D_DtN.py)."""
    dev = st._device(device)
    coeffs = _leaf_coefficients(pde_problem, dev)
    Y, T, v, h = st._local_solve_dtn(pde_problem, pde_problem.P, pde_problem.Q, dev, dtype, False,
                                     coefficients=coeffs)
    inv_h = torch.as_tensor(2.0 / np.asarray(pde_problem.sidelens, dtype=np.float64), device=dev)
    L = nat.lib()
    for x in (T, h):
        if x is not None:
            nat.check(L.hps_scale_batched(nat.TORCH_TO_HPS[x.dtype], x.shape[0], x[0].numel(), inv_h.data_ptr(),
                                          x.data_ptr(), nat.stream_ptr()), "hps_scale_batched")
    return Y, T, v, h


def _panel_map(mode, tab, M, src, ld_in, s_in, out, ld_out, s_out, batch, n_other, m_len):
    nat.check(nat.lib().hps_panel_map(nat.TORCH_TO_HPS[out.dtype], mode, batch, tab.shape[0], n_other, m_len,
                                      tab.data_ptr(), nat.ptr(M), src.data_ptr(), ld_in, s_in, out.data_ptr(), ld_out,
                                      s_out, nat.stream_ptr()), "hps_panel_map")


def _projection_ops(pde_problem, dtype, dev):
    """(rows compression, columns compression / expansion) matrices:
    (L_1f4, L_4f1) in 3D, (L_1f2, L_2f1) in 2D."""
    if pde_problem.domain.bool_2D:
        rows, cols = pde_problem.L_1f2, pde_problem.L_2f1
    else:
        rows, cols = pde_problem.L_1f4, pde_problem.L_4f1
    return (torch.as_tensor(np.ascontiguousarray(rows), dtype=dtype, device=dev),
            torch.as_tensor(np.ascontiguousarray(cols), dtype=dtype, device=dev))


def merge_stage_adaptive_3D_DtN(pde_problem, T_arr, h_arr, device=None, return_T: bool = False):
    """Bottom-up merges of an adaptive octree (or quadtree).  Stores S, g~,
    T, h in every internal node's ``data`` and the level buckets on the
    problem; returns the number of buckets."""
    dev = st._device(device)
    root = pde_problem.domain.root
    q = pde_problem.domain.q
    g = _geom(root)
    leaves = get_all_leaves(root)
    dtype = T_arr.dtype
    hh = None if h_arr is None else (h_arr if h_arr.dim() == 3 else h_arr.unsqueeze(-1))
    ns = 0 if hh is None else hh.shape[-1]
    for i, lf in enumerate(leaves):
        lf.data.T = T_arr[i]
        lf.data.h = None if hh is None else hh[i]
    L_rows, L_cols = _projection_ops(pde_problem, dtype, dev)
    plans: Dict[tuple, MergePlan] = {}
    levels: List[List[Bucket]] = []
    infos: list = []
    depth = get_depth(root)
    pan = q ** (g.dim - 1)
    K = g.nch
    for level in range(depth - 1, -1, -1):
        groups: Dict[tuple, list] = {}
        for node in get_nodes_at_level(root, level):
            if not len(node.children):
                continue
            sizes = tuple(_face_sizes(ch) for ch in node.children)
            proj = projection_lists(node)
            key = (sizes, tuple(sorted(proj.items())))
            groups.setdefault(key, []).append(node)
            if key not in plans:
                plans[key] = _build_plan(sizes, proj, q, dev, g)
        buckets = []
        for key, nodes in groups.items():
            plan = plans[key]
            nm, R = len(nodes), plan.nbr_max
            Tpad = torch.zeros((nm, K, R, R), dtype=dtype, device=dev)
            hpad = torch.zeros((nm, K, R, ns), dtype=dtype, device=dev) if ns else None
            for c in range(K):
                Tc = torch.stack([n.children[c].data.T for n in nodes])
                nb, nbr = plan.nb[c], plan.nbr[c]
                if plan.any_compressed[c]:
                    tmp = torch.empty((nm, nbr, nb), dtype=dtype, device=dev)
                    _panel_map(0, plan.compress[c], L_rows, Tc, nb, nb * nb, tmp, nb, nbr * nb, nm, nb, pan)
                    _panel_map(1, plan.compress[c], L_cols, tmp, nb, nbr * nb, Tpad[:, c], R, K * R * R, nm, nbr, pan)
                else:
                    Tpad[:, c, :nb, :nb] = Tc
                if ns:
                    hc = torch.stack([n.children[c].data.h for n in nodes])
                    if plan.any_compressed[c]:
                        _panel_map(0, plan.compress[c], L_rows, hc, ns, nb * ns, hpad[:, c], ns, K * R * ns, nm, ns,
                                   pan)
                    else:
                        hpad[:, c, :nb] = hc
            is_root = level == 0
            S, g_t, T_out, h_out, _, _ = st.merge_level_dtn(
                Tpad.view(nm * K, R, R), None if hpad is None else hpad.view(nm * K, R, ns), plan.maps,
                need_T=(not is_root) or return_T, infos=infos)
            for m, node in enumerate(nodes):
                node.data.S = S[m]
                node.data.g_tilde = None if g_t is None else g_t[m]
                node.data.T = None if T_out is None else T_out[m]
                node.data.h = None if h_out is None else h_out[m]
            buckets.append(Bucket(nodes, plan, S, g_t))
        levels.append(buckets)
    st.raise_on_sync_timeout(infos)
    levels.reverse()          # root level first
    pde_problem._adaptive_levels = levels
    return sum(len(b) for b in levels)


def down_pass_adaptive_3D_DtN(pde_problem, boundary_data, device=None, host_device=None):
    """Leaf solutions (n_leaves, p^d[, nsrc]) from Dirichlet data on the root
    boundary (a list of six face (3D) or four side (2D) arrays, or one array
    in the root's order)."""
    dev = st._device(device)
    root = pde_problem.domain.root
    q = pde_problem.domain.q
    g_ = _geom(root)
    K = g_.nch
    pan = q ** (g_.dim - 1)
    Y, v = pde_problem.Y, pde_problem.v
    dtype = Y.dtype
    if isinstance(boundary_data, (list, tuple)):
        parts = [b if isinstance(b, torch.Tensor) else torch.as_tensor(np.asarray(b)) for b in boundary_data]
        g = torch.cat([x.to(device=dev, dtype=dtype) for x in parts])
    else:
        g = st._as_tensor(boundary_data, dtype, dev)
    single = g.dim() == 1
    if single:
        g = g.unsqueeze(-1)
    ns = g.shape[-1]
    _, L_cols = _projection_ops(pde_problem, dtype, dev)
    root.data.g = g.contiguous()
    for buckets in pde_problem._adaptive_levels:
        for bk in buckets:
            plan = bk.plan
            nm, R = len(bk.nodes), plan.nbr_max
            gpar = torch.stack([n.data.g for n in bk.nodes])
            gt = bk.g_tilde
            if gt is not None and gt.shape[-1] != ns:
                gt = gt.expand(-1, -1, ns).contiguous()
            gch = st.down_level(bk.S, gt, gpar, plan.maps).view(nm, K, R, ns)
            for c in range(K):
                nb, nbr = plan.nb[c], plan.nbr[c]
                if plan.any_compressed[c]:
                    out = torch.empty((nm, nb, ns), dtype=dtype, device=dev)
                    _panel_map(0, plan.expand[c], L_cols, gch[:, c], ns, K * R * ns, out, ns, nb * ns, nm, ns, pan)
                else:
                    out = gch[:, c, :nb].contiguous()
                for m, node in enumerate(bk.nodes):
                    node.children[c].data.g = out[m]
    leaves = get_all_leaves(root)
    gl = torch.stack([lf.data.g for lf in leaves]).contiguous()
    u = torch.empty((Y.shape[0], Y.shape[1], ns), dtype=dtype, device=dev)
    if v is not None:
        vv = v if v.dim() == 3 else v.unsqueeze(-1)
        if vv.shape[-1] != ns:
            vv = vv.expand(-1, -1, ns)
        nat.gemm(Y, gl, u, 1.0, 1.0, Cmat=vv.contiguous())
    else:
        nat.gemm(Y, gl, u)
    for i, lf in enumerate(leaves):
        lf.data.u = u[i]
    if single and (v is None or v.dim() == 2):
        u = u[..., 0]
    return st._to_host(u, host_device)


def adaptive_build_solver(pde_problem, return_top_T=False, device=None, dtype=torch.float64):
    """_build_solver.py:177-258 for adaptive octrees and quadtrees (DtN)."""
    dom = pde_problem.domain
    if pde_problem.use_ItI:
        raise NotImplementedError("ItI merges are not supported for adaptive problems.")
    Y, T, v, h = local_solve_stage_adaptive_3D_DtN(pde_problem, device=device, dtype=dtype)
    pde_problem.Y, pde_problem.v = Y, v
    for i, lf in enumerate(get_all_leaves(dom.root)):
        lf.data.Y = Y[i]
        lf.data.v = None if v is None else v[i]
    merge_stage_adaptive_3D_DtN(pde_problem, T, h, device=device, return_T=return_top_T)
    if return_top_T:
        return dom.root.data.T
    return None


def adaptive_solve(pde_problem, boundary_data, device=None, host_device="cpu"):
    """_solve.py:96-112 for adaptive octrees and quadtrees."""
    return down_pass_adaptive_3D_DtN(pde_problem, boundary_data, device=device, host_device=host_device)


# 2D names of the same stages (local_solve/_adaptive_2D_DtN.py,
# merge/_adaptive_2D_DtN.py:24-117, down_pass/_adaptive_2D_DtN.py)
local_solve_stage_adaptive_2D_DtN = local_solve_stage_adaptive_3D_DtN
merge_stage_adaptive_2D_DtN = merge_stage_adaptive_3D_DtN
down_pass_adaptive_2D_DtN = down_pass_adaptive_3D_DtN


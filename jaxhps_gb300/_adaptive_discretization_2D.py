"""Adaptive quadtree generation (mirror of src/jaxhps/_adaptive_discretization_2D.py).

``generate_adaptive_mesh_level_restriction_2D`` refines a tree until every
leaf resolves f to ``tol``: a queued node is refined when interpolating f
from the node's Chebyshev grid to its four children's grids misses the
values of f there by ``tol`` (relative L-infinity, or relative squared L2
with ``l2_norm``), followed by 2:1 level restriction (:34-197).  The tree
edits run on the host; each round's point generation, f evaluation and
interpolation check run batched on the GPU (hps_refine_points_2d,
hps_refine_check_2d).  f is called as for the 3D meshing
(``_adaptive_discretization_3D.evaluate_f``).
"""

from __future__ import annotations

import time
from typing import Callable, List

import numpy as np
import torch

from . import _native as nat
from ._adaptive_discretization_3D import _close, evaluate_f
from ._discretization_tree import DiscretizationNode2D, get_all_leaves
from ._discretization_tree_operations_2D import add_four_children
from ._grid_creation_2D import (
    compute_interior_Chebyshev_points_adaptive_2D,
    compute_interior_Chebyshev_points_uniform_2D,
    rearrange_indices_ext_int,
)
from ._quadrature import (
    affine_transform,
    barycentric_lagrange_interpolation_matrix_1D,
    chebyshev_points,
    chebyshev_weights,
)

NODE_BATCH = 16384   # nodes per GPU check launch (points: NODE_BATCH * 5 p^2 * 16 bytes)


def node_to_bounds(node: DiscretizationNode2D) -> np.ndarray:
    return np.array(node.bounds)


class _CheckConstants2D:
    def __init__(self, p: int, dev):
        c = chebyshev_points(p)
        r = rearrange_indices_ext_int(p)
        ir = np.empty_like(r)
        ir[r] = np.arange(p ** 2)
        self.p = p
        self.cheb = torch.as_tensor(c, device=dev)
        self.perm = torch.as_tensor(r.astype(np.int32), device=dev)
        self.iperm = torch.as_tensor(ir.astype(np.int32), device=dev)
        self.Ilo = torch.as_tensor(barycentric_lagrange_interpolation_matrix_1D(c, affine_transform(c, (-1.0, 0.0))),
                                   device=dev).contiguous()
        self.Ihi = torch.as_tensor(barycentric_lagrange_interpolation_matrix_1D(c, affine_transform(c, (0.0, 1.0))),
                                   device=dev).contiguous()
        self.wref = torch.as_tensor(chebyshev_weights(p, (-1.0, 1.0)), device=dev)


def refinement_points_2d(bounds: np.ndarray, consts: _CheckConstants2D, dev) -> torch.Tensor:
    """(n, 5, p^2, 2): every node's grid followed by its children's grids."""
    L = nat.lib()
    p = consts.p
    b = torch.as_tensor(np.ascontiguousarray(bounds, dtype=np.float64), device=dev)
    pts = torch.empty((b.shape[0], 5, p ** 2, 2), dtype=torch.float64, device=dev)
    nat.check(L.hps_refine_points_2d(b.shape[0], p, b.data_ptr(), consts.cheb.data_ptr(), consts.perm.data_ptr(),
                                     pts.data_ptr(), nat.stream_ptr()), "hps_refine_points_2d")
    return pts


def refinement_check_2d(bounds: np.ndarray, f_fn: Callable, consts: _CheckConstants2D, dev, want_l2: bool = False):
    """(diff_max, ref_max, l2) per node, NumPy arrays (l2 None unless asked)."""
    L = nat.lib()
    p = consts.p
    n = bounds.shape[0]
    diff = torch.empty(n, dtype=torch.float64, device=dev)
    ref = torch.empty(n, dtype=torch.float64, device=dev)
    l2 = torch.empty(n, dtype=torch.float64, device=dev) if want_l2 else None
    for s in range(0, n, NODE_BATCH):
        bb = bounds[s:s + NODE_BATCH]
        pts = refinement_points_2d(bb, consts, dev)
        fv = evaluate_f(f_fn, pts).reshape(bb.shape[0], 5, p ** 2).contiguous()
        btd = torch.as_tensor(np.ascontiguousarray(bb, dtype=np.float64), device=dev)
        nat.check(L.hps_refine_check_2d(bb.shape[0], p, fv.data_ptr(), consts.perm.data_ptr(), consts.iperm.data_ptr(),
                                        consts.Ilo.data_ptr(), consts.Ihi.data_ptr(), consts.wref.data_ptr(),
                                        btd.data_ptr(), diff[s:].data_ptr(), ref[s:].data_ptr(),
                                        None if l2 is None else l2[s:].data_ptr(), nat.stream_ptr()),
                  "hps_refine_check_2d")
    return diff.cpu().numpy(), ref.cpu().numpy(), (None if l2 is None else l2.cpu().numpy())


def get_squared_l2_norm_single_panel(f_evals: np.ndarray, bounds, p: int) -> float:
    """Clenshaw-Curtis squared L2 norm of f on one leaf grid (:380-407)."""
    w = np.outer(chebyshev_weights(p, bounds[:2]), chebyshev_weights(p, bounds[2:])).ravel()[
        rearrange_indices_ext_int(p)]
    return float(np.sum(w * np.asarray(f_evals) ** 2))


def patches_to_check(newly_refined: DiscretizationNode2D, root: DiscretizationNode2D) -> np.ndarray:
    """Same-size patches side-adjacent to a newly refined node (:200-277)."""
    n = newly_refined
    s = n.xmax - n.xmin
    vols = []
    if n.xmin - s >= root.xmin:
        vols.append([n.xmin - s, n.xmin, n.ymin, n.ymax])
    if n.xmax + s <= root.xmax:
        vols.append([n.xmax, n.xmax + s, n.ymin, n.ymax])
    if n.ymin - s >= root.ymin:
        vols.append([n.xmin, n.xmax, n.ymin - s, n.ymin])
    if n.ymax + s <= root.ymax:
        vols.append([n.xmin, n.xmax, n.ymax, n.ymax + s])
    return np.array(vols)


def find_or_add_child_2D(node: DiscretizationNode2D, root: DiscretizationNode2D, q: int, xmin: float, xmax: float,
                         ymin: float, ymax: float):
    """Makes sure the tree resolves the patch at half its size: refines the
    node holding it if that node is a leaf and returns it, else None
    (:280-352)."""
    while True:
        side = node.xmax - node.xmin
        req = xmax - xmin
        if _close(req * 2, side):
            if not len(node.children):
                add_four_children(node, root=root, q=q)
                return node
            return None
        xm, ym = (node.xmax + node.xmin) / 2, (node.ymax + node.ymin) / 2
        if xmin < xm:
            c = 0 if ymin < ym else 3
        else:
            c = 1 if ymin < ym else 2
        child = node.children[c]
        if _close(side, 4 * req):
            if not len(child.children):
                add_four_children(child, root=root, q=q)
                return child
            return None
        if side < 2 * req:
            raise ValueError("Requested volume is too large for the current node")
        node = child


def generate_adaptive_mesh_level_restriction_2D(root: DiscretizationNode2D, f_fn: Callable, tol: float, p: int,
                                                q: int, restrict_bool: bool = True, l2_norm: bool = False,
                                                device=None, stats: dict | None = None) -> None:
    """Refines ``root`` in place (:34-197)."""
    t0 = time.perf_counter()
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    nat.lib()
    consts = _CheckConstants2D(p, dev)
    if l2_norm:
        add_four_children(root, root=root, q=q)
        leaves = get_all_leaves(root)
        pts = torch.as_tensor(compute_interior_Chebyshev_points_adaptive_2D(root, p), device=dev)
        fv = evaluate_f(f_fn, pts).cpu().numpy()
        global_nrm = sum(get_squared_l2_norm_single_panel(fv[i], np.array(lf.bounds), p)
                         for i, lf in enumerate(leaves))
        tol = tol ** 2
    else:
        pts1 = torch.as_tensor(compute_interior_Chebyshev_points_uniform_2D(root, 1, p).reshape(-1, 2), device=dev)
        # the reference takes the signed maximum here (:70)
        global_nrm = float(evaluate_f(f_fn, pts1).max().item())
    queue: List[DiscretizationNode2D] = list(get_all_leaves(root))
    n_rounds = n_checked = 0
    while queue:
        n_rounds += 1
        bounds = np.array([nd.bounds for nd in queue])
        diff, ref, l2 = refinement_check_2d(bounds, f_fn, consts, dev, want_l2=l2_norm)
        n_checked += len(queue)
        if l2_norm:
            fails = ~(l2 / global_nrm < tol)
        else:
            nrm = np.maximum(global_nrm, ref)
            fails = ~(diff / nrm < tol)
            global_nrm = float(nrm.max())
        new_queue: List[DiscretizationNode2D] = []
        for i, node in enumerate(queue):
            if not fails[i]:
                continue
            add_four_children(node, root=root, q=q)
            new_queue.extend(node.children)
            if restrict_bool:
                pending = [node]
                while pending:
                    for_check = pending.pop()
                    for vol in patches_to_check(for_check, root):
                        n = find_or_add_child_2D(root, root, q, *vol)
                        if n is not None:
                            pending.append(n)
                            new_queue.extend(n.children)
        queue = new_queue
    if stats is not None:
        stats.update(rounds=n_rounds, checked=n_checked, seconds=time.perf_counter() - t0,
                     leaves=len(get_all_leaves(root)), global_norm=global_nrm, tol=tol)

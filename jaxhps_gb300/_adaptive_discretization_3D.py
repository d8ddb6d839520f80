"""Adaptive octree generation (mirror of src/jaxhps/_adaptive_discretization_3D.py).

``generate_adaptive_mesh_level_restriction`` refines a tree until every leaf
resolves f to ``tol``: a queued node is refined when interpolating f from
the node's Chebyshev grid to its eight children's grids misses the values of
f there by ``tol`` (relative L-infinity, or relative squared L2 with
``l2_norm``), followed by 2:1 level restriction (:34-210).  The tree edits
run on the host; each round's point generation, f evaluation and
interpolation check run batched on the GPU (hps_refine_points_3d,
hps_refine_check_3d).

f is called with a torch tensor of points (..., 3) on the compute device;
if it does not return a torch tensor (or raises), it is called with a NumPy
array on the host instead.

An optional ``proposer`` (``jaxhps_gb300.refinement_mlp.RefinementProposer``)
predicts refine/keep for queued nodes from cheap samples of f; nodes it
marks as "refine" with high confidence are refined without the full check,
every other node — in particular every node that ends as a leaf — is
decided by the plain criterion above.
"""

from __future__ import annotations

import time
from typing import Callable, List

import numpy as np
import torch

from . import _native as nat
from ._discretization_tree import DiscretizationNode3D, get_all_leaves
from ._discretization_tree_operations_3D import add_eight_children
from ._grid_creation_3D import (
    compute_interior_Chebyshev_points_adaptive_3D,
    compute_interior_Chebyshev_points_uniform_3D,
    rearrange_indices_ext_int,
)
from ._quadrature import (
    affine_transform,
    barycentric_lagrange_interpolation_matrix_1D,
    chebyshev_points,
    chebyshev_weights,
)

NODE_BATCH = 4096   # nodes per GPU check launch (points: NODE_BATCH * 9 p^3 * 24 bytes)


def node_to_bounds(node: DiscretizationNode3D) -> np.ndarray:
    return np.array(node.bounds)


def evaluate_f(f_fn: Callable, pts: torch.Tensor) -> torch.Tensor:
    """f at points (..., 3): on the device when f handles torch tensors,
    otherwise through NumPy on the host."""
    try:
        out = f_fn(pts)
        if isinstance(out, torch.Tensor):
            return out.to(device=pts.device, dtype=torch.float64)
    except Exception:
        pass
    out = np.asarray(f_fn(pts.detach().cpu().numpy()), dtype=np.float64)
    return torch.as_tensor(out, device=pts.device)


class _CheckConstants:
    def __init__(self, p: int, dev):
        c = chebyshev_points(p)
        r = rearrange_indices_ext_int(p)
        ir = np.empty_like(r)
        ir[r] = np.arange(p ** 3)
        lo = affine_transform(c, (-1.0, 0.0))
        hi = affine_transform(c, (0.0, 1.0))
        self.p = p
        self.cheb = torch.as_tensor(c, device=dev)
        self.perm = torch.as_tensor(r.astype(np.int32), device=dev)
        self.iperm = torch.as_tensor(ir.astype(np.int32), device=dev)
        self.Ilo = torch.as_tensor(barycentric_lagrange_interpolation_matrix_1D(c, lo), device=dev).contiguous()
        self.Ihi = torch.as_tensor(barycentric_lagrange_interpolation_matrix_1D(c, hi), device=dev).contiguous()
        self.wref = torch.as_tensor(chebyshev_weights(p, (-1.0, 1.0)), device=dev)


def refinement_points(bounds: np.ndarray, consts: _CheckConstants, dev) -> torch.Tensor:
    """(n, 9, p^3, 3): every node's grid followed by its children's grids."""
    L = nat.lib()
    p = consts.p
    b = torch.as_tensor(np.ascontiguousarray(bounds, dtype=np.float64), device=dev)
    pts = torch.empty((b.shape[0], 9, p ** 3, 3), dtype=torch.float64, device=dev)
    nat.check(L.hps_refine_points_3d(b.shape[0], p, b.data_ptr(), consts.cheb.data_ptr(), consts.perm.data_ptr(),
                                     pts.data_ptr(), nat.stream_ptr()), "hps_refine_points_3d")
    return pts


def refinement_check(bounds: np.ndarray, f_fn: Callable, consts: _CheckConstants, dev, want_l2: bool = False):
    """(diff_max, ref_max, l2) per node, NumPy arrays (l2 None unless asked)."""
    L = nat.lib()
    p = consts.p
    n = bounds.shape[0]
    diff = torch.empty(n, dtype=torch.float64, device=dev)
    ref = torch.empty(n, dtype=torch.float64, device=dev)
    l2 = torch.empty(n, dtype=torch.float64, device=dev) if want_l2 else None
    for s in range(0, n, NODE_BATCH):
        bb = bounds[s:s + NODE_BATCH]
        pts = refinement_points(bb, consts, dev)
        fv = evaluate_f(f_fn, pts).reshape(bb.shape[0], 9, p ** 3).contiguous()
        btd = torch.as_tensor(np.ascontiguousarray(bb, dtype=np.float64), device=dev)
        nat.check(L.hps_refine_check_3d(bb.shape[0], p, fv.data_ptr(), consts.perm.data_ptr(), consts.iperm.data_ptr(),
                                        consts.Ilo.data_ptr(), consts.Ihi.data_ptr(), consts.wref.data_ptr(),
                                        btd.data_ptr(), diff[s:].data_ptr(), ref[s:].data_ptr(),
                                        None if l2 is None else l2[s:].data_ptr(), nat.stream_ptr()),
                  "hps_refine_check_3d")
    return diff.cpu().numpy(), ref.cpu().numpy(), (None if l2 is None else l2.cpu().numpy())


def get_squared_l2_norm_single_voxel(f_evals: np.ndarray, bounds, p: int) -> float:
    """Clenshaw-Curtis squared L2 norm of f on one leaf grid (:446-472)."""
    w = np.einsum("i,j,k->ijk", chebyshev_weights(p, bounds[:2]), chebyshev_weights(p, bounds[2:4]),
                  chebyshev_weights(p, bounds[4:])).ravel()[rearrange_indices_ext_int(p)]
    return float(np.sum(w * np.asarray(f_evals) ** 2))


def check_current_discretization_global_linf_norm(f_evals, f_evals_refined, refinement_op, tol: float,
                                                  global_linf_norm: float):
    """Dense form of the L-infinity check (:475-503): (passes, norm constant)."""
    f_interp = refinement_op @ f_evals
    ref_max = np.max(np.abs(f_evals_refined))
    nrm = max(global_linf_norm, ref_max)
    return np.max(np.abs(f_interp - f_evals_refined)) / nrm < tol, nrm


def volumes_to_check(newly_refined: DiscretizationNode3D, root: DiscretizationNode3D) -> np.ndarray:
    """Same-size volumes face-adjacent to a newly refined node (:213-314)."""
    n = newly_refined
    s = n.xmax - n.xmin
    vols = []
    if n.xmin - s >= root.xmin:
        vols.append([n.xmin - s, n.xmin, n.ymin, n.ymax, n.zmin, n.zmax])
    if n.xmax + s <= root.xmax:
        vols.append([n.xmax, n.xmax + s, n.ymin, n.ymax, n.zmin, n.zmax])
    if n.ymin - s >= root.ymin:
        vols.append([n.xmin, n.xmax, n.ymin - s, n.ymin, n.zmin, n.zmax])
    if n.ymax + s <= root.ymax:
        vols.append([n.xmin, n.xmax, n.ymax, n.ymax + s, n.zmin, n.zmax])
    if n.zmin - s >= root.zmin:
        vols.append([n.xmin, n.xmax, n.ymin, n.ymax, n.zmin - s, n.zmin])
    if n.zmax + s <= root.zmax:
        vols.append([n.xmin, n.xmax, n.ymin, n.ymax, n.zmax, n.zmax + s])
    return np.array(vols)


def _close(a: float, b: float) -> bool:
    # numpy.allclose defaults, as jnp.allclose in the reference
    return abs(a - b) <= 1e-8 + 1e-5 * abs(b)


def find_or_add_child(node: DiscretizationNode3D, root: DiscretizationNode3D, q: int, xmin: float, xmax: float,
                      ymin: float, ymax: float, zmin: float, zmax: float):
    """Makes sure the tree resolves the volume at half its size: refines the
    node holding it if that node is a leaf and returns it, else None
    (:317-420)."""
    while True:
        side = node.xmax - node.xmin
        req = xmax - xmin
        if _close(req * 2, side):
            if not len(node.children):
                add_eight_children(node, root=root, q=q)
                return node
            return None
        xm, ym, zm = (node.xmax + node.xmin) / 2, (node.ymax + node.ymin) / 2, (node.zmax + node.zmin) / 2
        if xmin < xm:
            c = (4 if zmin < zm else 0) if ymin < ym else (7 if zmin < zm else 3)
        else:
            c = (5 if zmin < zm else 1) if ymin < ym else (6 if zmin < zm else 2)
        child = node.children[c]
        if _close(side, 4 * req):
            if not len(child.children):
                add_eight_children(child, root=root, q=q)
                return child
            return None
        if side < 2 * req:
            raise ValueError("Requested volume is too large for the current node")
        node = child


def generate_adaptive_mesh_level_restriction(root: DiscretizationNode3D, f_fn: Callable, tol: float, p: int, q: int,
                                             restrict_bool: bool = True, l2_norm: bool = False, proposer=None,
                                             device=None, stats: dict | None = None) -> None:
    """Refines ``root`` in place (:34-210).  ``stats`` (optional dict) receives
    the number of rounds, of fully checked nodes, of nodes refined on the
    proposer's word, the wall time, and the wall time per phase summed over
    the rounds (``t_propose``: the proposer's features and network;
    ``t_check``: f at the check points and the batched criterion on the GPU,
    with the device sync that returns its verdicts; ``t_edit``: the host-side
    tree edits, level restriction included) with the same split per round in
    ``rounds_detail``."""
    t0 = time.perf_counter()
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    nat.lib()
    consts = _CheckConstants(p, dev)
    if l2_norm:
        add_eight_children(root, root=root, q=q)
        leaves = get_all_leaves(root)
        pts = torch.as_tensor(compute_interior_Chebyshev_points_adaptive_3D(root, p), device=dev)
        fv = evaluate_f(f_fn, pts).cpu().numpy()
        global_nrm = sum(get_squared_l2_norm_single_voxel(fv[i], np.array(lf.bounds), p)
                         for i, lf in enumerate(leaves))
        tol = tol ** 2
    else:
        pts1 = torch.as_tensor(compute_interior_Chebyshev_points_uniform_3D(root, 1, p).reshape(-1, 3), device=dev)
        # the reference takes the signed maximum here (:70)
        global_nrm = float(evaluate_f(f_fn, pts1).max().item())
    queue: List[DiscretizationNode3D] = list(get_all_leaves(root))
    n_rounds = n_checked = n_proposed = 0
    detail = []
    while queue:
        n_rounds += 1
        ta = time.perf_counter()
        to_refine = np.zeros(len(queue), dtype=bool)
        check_idx = np.arange(len(queue))
        if proposer is not None:
            sure = proposer.confident_refine(queue, f_fn, global_nrm, dev)
            to_refine |= sure
            n_proposed += int(sure.sum())
            check_idx = np.nonzero(~sure)[0]
        tb = time.perf_counter()
        if len(check_idx):
            bounds = np.array([queue[i].bounds for i in check_idx])
            diff, ref, l2 = refinement_check(bounds, f_fn, consts, dev, want_l2=l2_norm)
            n_checked += len(check_idx)
            if l2_norm:
                fails = ~(l2 / global_nrm < tol)
            else:
                nrm = np.maximum(global_nrm, ref)
                fails = ~(diff / nrm < tol)
                global_nrm = float(nrm.max())
            to_refine[check_idx] = fails
            if proposer is not None:
                proposer.record(queue, check_idx, fails)
        tc = time.perf_counter()
        new_queue: List[DiscretizationNode3D] = []
        for i, node in enumerate(queue):
            if not to_refine[i]:
                continue
            add_eight_children(node, root=root, q=q)
            new_queue.extend(node.children)
            if restrict_bool:
                pending = [node]
                while pending:
                    for_check = pending.pop()
                    for vol in volumes_to_check(for_check, root):
                        n = find_or_add_child(root, root, q, *vol)
                        if n is not None:
                            pending.append(n)
                            new_queue.extend(n.children)
        detail.append(dict(queued=len(queue), checked=int(len(check_idx)), refined=int(to_refine.sum()),
                           t_propose=tb - ta, t_check=tc - tb, t_edit=time.perf_counter() - tc))
        queue = new_queue
    if stats is not None:
        stats.update(rounds=n_rounds, checked=n_checked, proposed=n_proposed, seconds=time.perf_counter() - t0,
                     leaves=len(get_all_leaves(root)), global_norm=global_nrm, tol=tol, rounds_detail=detail,
                     **{k: sum(d[k] for d in detail) for k in ("t_propose", "t_check", "t_edit")})

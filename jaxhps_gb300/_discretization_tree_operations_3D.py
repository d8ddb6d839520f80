"""Octree editing (host side), mirroring src/jaxhps/_discretization_tree_operations_3D.py.

Children are a..h (a-d upper z half; each half (x lo, y lo), (x hi, y lo),
(x hi, y hi), (x lo, y hi)).  ``n_0 .. n_5`` count the Gauss points on a
node's faces -x, +x, -y, +y, -z, +z; they are kept current while the tree is
refined (:57-98), as the adaptive merges size their blocks from them.
"""

from __future__ import annotations

from typing import List, Tuple

from ._discretization_tree import DiscretizationNode3D, get_all_leaves
from ._grid_creation_3D import bounds_for_oct_subdivision, get_all_leaves_special_ordering_3D  # noqa: F401


def get_eight_children(parent: DiscretizationNode3D) -> Tuple[DiscretizationNode3D, ...]:
    return tuple(DiscretizationNode3D(*b, depth=parent.depth + 1) for b in bounds_for_oct_subdivision(parent.bounds))


def tree_equal(node_a, node_b) -> bool:
    """Same bounds, depth and tree shape (the reference compares pytree
    structures, :340-346)."""
    if node_a is node_b:
        return True
    if node_a.bounds != node_b.bounds or node_a.depth != node_b.depth or len(node_a.children) != len(node_b.children):
        return False
    return all(tree_equal(a, b) for a, b in zip(node_a.children, node_b.children))


def _child_index(node, x0: float, y0: float, z0: float) -> int:
    """Index (a..h = 0..7) of node's child containing the lower corner (x0, y0, z0)."""
    xm = (node.xmin + node.xmax) / 2
    ym = (node.ymin + node.ymax) / 2
    zm = (node.zmin + node.zmax) / 2
    quad = (0, 3) if x0 < xm else (1, 2)
    c = quad[0] if y0 < ym else quad[1]
    return c + 4 if z0 < zm else c


def find_path_from_root_3D(root: DiscretizationNode3D, node: DiscretizationNode3D) -> List[DiscretizationNode3D]:
    """Ancestors of ``node`` from the root down to its parent (:212-271)."""
    if not len(root.children):
        raise ValueError("Specified root has no children.")
    path = []
    cur = root
    while True:
        path.append(cur)
        if any(ch is node or tree_equal(ch, node) for ch in cur.children):
            return path
        nxt = cur.children[_child_index(cur, node.xmin, node.ymin, node.zmin)]
        if not len(nxt.children):
            raise ValueError("node is not in the tree")
        cur = nxt


def add_eight_children(add_to: DiscretizationNode3D, root: DiscretizationNode3D = None, q: int = None) -> None:
    """Splits a leaf into its children a..h; with ``root`` and ``q`` also
    updates the face point counts of the node and of every ancestor sharing
    a face with it (:26-98).  A node that already has children is left
    unchanged."""
    if len(add_to.children):
        return
    add_to.children = get_eight_children(add_to)
    if q is None:
        return
    q2 = q * q
    for ch in add_to.children:
        ch.n_0 = ch.n_1 = ch.n_2 = ch.n_3 = ch.n_4 = ch.n_5 = q2
    add_to.n_0 = add_to.n_1 = add_to.n_2 = add_to.n_3 = add_to.n_4 = add_to.n_5 = 4 * q2
    if root is None or add_to is root or tree_equal(add_to, root):
        return
    for node in find_path_from_root_3D(root, add_to):
        if node.xmin == add_to.xmin:
            node.n_0 += 3 * q2
        if node.xmax == add_to.xmax:
            node.n_1 += 3 * q2
        if node.ymin == add_to.ymin:
            node.n_2 += 3 * q2
        if node.ymax == add_to.ymax:
            node.n_3 += 3 * q2
        if node.zmin == add_to.zmin:
            node.n_4 += 3 * q2
        if node.zmax == add_to.zmax:
            node.n_5 += 3 * q2


def find_nodes_along_interface_3D(root: DiscretizationNode3D, xval: float = None, yval: float = None,
                                  zval: float = None):
    """Leaves bordering the plane x = xval (or y, z): (negative side, positive side) (:274-337)."""
    if sum(v is not None for v in (xval, yval, zval)) != 1:
        raise ValueError(f"Only one of xval, yval, or zval can be specified. Input args: {xval}, {yval}, {zval}")
    lo, hi, val = (("xmin", "xmax", xval) if xval is not None else
                   ("ymin", "ymax", yval) if yval is not None else ("zmin", "zmax", zval))
    neg, pos = [], []
    for leaf in get_all_leaves(root):
        if getattr(leaf, lo) == val:
            pos.append(leaf)
        elif getattr(leaf, hi) == val:
            neg.append(leaf)
    return neg, pos

"""Quadtree editing (host side), mirroring src/jaxhps/_discretization_tree_operations_2D.py.

Children are a, b, c, d = SW, SE, NE, NW.  ``n_0 .. n_3`` count the Gauss
points on a node's sides S, E, N, W; they are kept current while the tree is
refined (:51-104), as the adaptive merges size their blocks from them.
"""

from __future__ import annotations

from typing import List, Optional, Tuple

from ._discretization_tree import DiscretizationNode2D
from ._grid_creation_2D import bounds_for_quad_subdivision


def get_four_children(parent: DiscretizationNode2D) -> Tuple[DiscretizationNode2D, ...]:
    return tuple(DiscretizationNode2D(*b, depth=parent.depth + 1) for b in bounds_for_quad_subdivision(parent.bounds))


def tree_equal(node_a, node_b) -> bool:
    """Same bounds, depth and tree shape (the reference compares pytree
    structures, :349-358)."""
    if node_a is node_b:
        return True
    if node_a.bounds != node_b.bounds or node_a.depth != node_b.depth or len(node_a.children) != len(node_b.children):
        return False
    return all(tree_equal(a, b) for a, b in zip(node_a.children, node_b.children))


def _child_index(node, x0: float, y0: float) -> int:
    """Index (a..d = 0..3) of node's child containing the lower corner (x0, y0)."""
    xm = (node.xmin + node.xmax) / 2
    ym = (node.ymin + node.ymax) / 2
    if x0 < xm:
        return 0 if y0 < ym else 3
    return 1 if y0 < ym else 2


def find_path_from_root_2D(root: DiscretizationNode2D, node: DiscretizationNode2D) -> List[DiscretizationNode2D]:
    """Ancestors of ``node`` from the root down to its parent (:107-153)."""
    if not len(root.children):
        raise ValueError("Specified root has no children.")
    path = []
    cur = root
    while True:
        path.append(cur)
        if any(ch is node or tree_equal(ch, node) for ch in cur.children):
            return path
        nxt = cur.children[_child_index(cur, node.xmin, node.ymin)]
        if not len(nxt.children):
            raise ValueError("node is not in the tree")
        cur = nxt


def add_four_children(add_to: DiscretizationNode2D, root: Optional[DiscretizationNode2D] = None,
                      q: Optional[int] = None) -> None:
    """Splits a leaf into its children a..d; with ``root`` and ``q`` also
    updates the side point counts of the node and of every ancestor sharing
    a side with it (:51-104).  A node that already has children is left
    unchanged."""
    if len(add_to.children):
        return
    add_to.children = get_four_children(add_to)
    if q is None:
        return
    for ch in add_to.children:
        ch.n_0 = ch.n_1 = ch.n_2 = ch.n_3 = q
    add_to.n_0 = add_to.n_1 = add_to.n_2 = add_to.n_3 = 2 * q
    if root is None or tree_equal(add_to, root):
        return
    for node in find_path_from_root_2D(root, add_to):
        if node.ymin == add_to.ymin:
            node.n_0 += q
        if node.xmax == add_to.xmax:
            node.n_1 += q
        if node.ymax == add_to.ymax:
            node.n_2 += q
        if node.xmin == add_to.xmin:
            node.n_3 += q


def node_at(node, xmin=None, xmax=None, ymin=None, ymax=None) -> bool:
    """Whether the node's bounds match every given value (:335-346)."""
    return ((xmin is None or node.xmin == xmin) and (xmax is None or node.xmax == xmax)
            and (ymin is None or node.ymin == ymin) and (ymax is None or node.ymax == ymax))


def find_node_at_corner(root: DiscretizationNode2D, xmin=None, xmax=None, ymin=None, ymax=None) -> DiscretizationNode2D:
    """The leaf with the given bounds values (the leaf at that corner or along
    that edge) (:276-332)."""
    node = root
    while True:
        if node_at(node, xmin, xmax, ymin, ymax):
            if not len(node.children):
                return node
            nxt = None
            for ch in node.children:
                if node_at(ch, xmin, xmax, ymin, ymax):
                    nxt = ch
                    break
            if nxt is None:
                return node
            node = nxt
            continue
        xm = (node.xmin + node.xmax) / 2
        ym = (node.ymin + node.ymax) / 2
        upper_x = (xmin is None or xmin >= xm) and (xmax is None or xmax > xm)
        upper_y = (ymin is None or ymin >= ym) and (ymax is None or ymax > ym)
        if upper_x:
            node = node.children[2] if upper_y else node.children[1]
        else:
            node = node.children[3] if upper_y else node.children[0]


def get_ordered_lst_of_boundary_nodes(root: DiscretizationNode2D) -> Tuple[Tuple[DiscretizationNode2D, ...], ...]:
    """Leaves along the S (W->E), E (S->N), N (E->W) and W (N->S) sides of
    the tree rooted at ``root`` (:156-273)."""
    s = [find_node_at_corner(root, xmin=root.xmin, ymin=root.ymin)]
    while s[-1].xmax != root.xmax:
        s.append(find_node_at_corner(root, xmin=s[-1].xmax, ymin=root.ymin))
    e = [s[-1]]
    while e[-1].ymax != root.ymax:
        e.append(find_node_at_corner(root, xmax=root.xmax, ymin=e[-1].ymax))
    n = [e[-1]]
    while n[-1].xmin != root.xmin:
        n.append(find_node_at_corner(root, xmax=n[-1].xmin, ymax=root.ymax))
    w = [n[-1]]
    while w[-1].ymin != root.ymin:
        w.append(find_node_at_corner(root, xmin=root.xmin, ymax=w[-1].ymin))
    return tuple(s), tuple(e), tuple(n), tuple(w)

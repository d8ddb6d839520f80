"""Discretization tree nodes (API mirror of src/jaxhps/_discretization_tree.py).

``DiscretizationNode2D`` / ``DiscretizationNode3D`` carry the box bounds,
depth, children and a ``NodeData`` container, exactly as in the reference
(:6-264).  Children of a 2D node are ordered SW, SE, NE, NW
(_grid_creation_2D.py:34-46).
"""

from __future__ import annotations

from typing import Tuple


class NodeData:
    """Per-node solver state (reference _discretization_tree.py:6-37)."""

    def __init__(self):
        self.T = None
        self.h = None
        self.S = None
        self.g_tilde = None
        self.Y = None
        self.v = None
        self.u = None
        self.g = None
        self.L_4f1 = None
        self.L_1f4 = None
        self.l2_nrm: float = 0.0


class DiscretizationNode2D:
    def __init__(self, xmin: float, xmax: float, ymin: float, ymax: float, depth: int = 0,
                 children: Tuple["DiscretizationNode2D", ...] = ()):
        self.xmin = float(xmin)
        self.xmax = float(xmax)
        self.ymin = float(ymin)
        self.ymax = float(ymax)
        self.depth = int(depth)
        self.data = NodeData()
        self.n_0 = None
        self.n_1 = None
        self.n_2 = None
        self.n_3 = None
        self.children = tuple(children)

    @property
    def bounds(self):
        return (self.xmin, self.xmax, self.ymin, self.ymax)

    def __repr__(self) -> str:
        return (f"DiscretizationNode2D(xmin={self.xmin}, xmax={self.xmax}, ymin={self.ymin}, "
                f"ymax={self.ymax}, depth={self.depth})")


class DiscretizationNode3D:
    def __init__(self, xmin: float, xmax: float, ymin: float, ymax: float, zmin: float, zmax: float,
                 depth: int = 0, children: Tuple["DiscretizationNode3D", ...] = ()):
        self.xmin = float(xmin)
        self.xmax = float(xmax)
        self.ymin = float(ymin)
        self.ymax = float(ymax)
        self.zmin = float(zmin)
        self.zmax = float(zmax)
        self.depth = int(depth)
        self.data = NodeData()
        self.n_0 = self.n_1 = self.n_2 = self.n_3 = self.n_4 = self.n_5 = None
        self.children = tuple(children)

    @property
    def bounds(self):
        return (self.xmin, self.xmax, self.ymin, self.ymax, self.zmin, self.zmax)

    def __repr__(self) -> str:
        return (f"DiscretizationNode3D(xmin={self.xmin}, xmax={self.xmax}, ymin={self.ymin}, "
                f"ymax={self.ymax}, zmin={self.zmin}, zmax={self.zmax}, depth={self.depth})")


def get_all_leaves(node):
    """All leaf descendants in depth-first child order (reference :276-295)."""
    if not len(node.children):
        return (node,)
    out = ()
    for c in node.children:
        out += get_all_leaves(c)
    return out


def get_depth(node) -> int:
    return max(leaf.depth for leaf in get_all_leaves(node))


def get_nodes_at_level(node, level: int):
    if node.depth == level:
        return (node,)
    out = ()
    for c in node.children:
        out += get_nodes_at_level(c, level)
    return out


def get_discretization_node_area(node) -> float:
    if isinstance(node, DiscretizationNode3D):
        return (node.xmax - node.xmin) * (node.ymax - node.ymin) * (node.zmax - node.zmin)
    return (node.xmax - node.xmin) * (node.ymax - node.ymin)

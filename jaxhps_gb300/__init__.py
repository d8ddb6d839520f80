"""jaxhps_gb300 — GB300-native HPS (hierarchical Poincare-Steklov) fast
direct solver with the public API of meliao/jaxhps:

    Domain, DiscretizationNode2D, DiscretizationNode3D, get_all_leaves,
    PDEProblem, build_solver, solve, solve_subtree, upward_pass_subtree,
    downward_pass_subtree

plus ``save_solver`` / ``load_solver`` (the built operator set as one file).

The leaf solves, merges and down pass run as hand-written sm_103a CUDA
kernels behind a C ABI (include/jaxhps_gb300.h); host code here only builds
the small FP64 operators, the index maps and the device buffers.
"""

from ._discretization_tree import (
    DiscretizationNode2D,
    DiscretizationNode3D,
    NodeData,
    get_all_leaves,
    get_depth,
    get_nodes_at_level,
)
from ._domain import Domain
from ._pdeproblem import PDEProblem
from ._build_solver import build_solver
from ._solve import solve
from ._subtree import downward_pass_subtree, solve_subtree, upward_pass_subtree
from ._checkpoint import load_solver, save_solver


def local_solve_chunksize_2D(p: int, dtype=None) -> int:
    """Leaf-stage chunk size.  The reference sizes chunks for an 80 GB GPU
    (_device_config.py:37-62); on a GB300 the leaves of trees up to 4^10
    (2D) / 8^6 (3D) leaves fit HBM at once, so the whole level is one chunk."""
    return 4 ** 10


def local_solve_chunksize_3D(p: int, dtype=None) -> int:
    return 8 ** 6


__all__ = [
    "Domain",
    "DiscretizationNode2D",
    "DiscretizationNode3D",
    "NodeData",
    "get_all_leaves",
    "get_depth",
    "get_nodes_at_level",
    "PDEProblem",
    "build_solver",
    "solve",
    "solve_subtree",
    "upward_pass_subtree",
    "downward_pass_subtree",
    "save_solver",
    "load_solver",
    "local_solve_chunksize_2D",
    "local_solve_chunksize_3D",
]
__version__ = "0.1.0"

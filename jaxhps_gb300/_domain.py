"""``Domain``: discretization of the computational box (API mirror of
src/jaxhps/_domain.py:38-97).

Holds p, q, the root node, the number of uniform levels L (None for an
adaptive tree), the leaf Chebyshev points ``interior_points``
(n_leaves, p^d, d) and the root boundary Gauss points ``boundary_points``.
Grid construction is host-side NumPy float64.
"""

from __future__ import annotations

from typing import Callable, List

import numpy as np

from ._discretization_tree import DiscretizationNode2D, get_all_leaves
from . import _grid_creation_2D as g2


class Domain:
    def __init__(self, p: int, q: int, root, L: int | None = None):
        self.p = int(p)
        self.q = int(q)
        self.root = root
        self.L = None if L is None else int(L)
        self.bool_2D = isinstance(root, DiscretizationNode2D)
        if self.L is not None:
            self.bool_uniform = True
            if self.bool_2D:
                self.interior_points = g2.compute_interior_Chebyshev_points_uniform_2D(root, self.L, self.p)
                self.boundary_points = g2.compute_boundary_Gauss_points_uniform_2D(root, self.L, self.q)
                self.n_leaves = 4 ** self.L
            else:
                from . import _grid_creation_3D as g3
                self.interior_points = g3.compute_interior_Chebyshev_points_uniform_3D(root, self.L, self.p)
                self.boundary_points = g3.compute_boundary_Gauss_points_uniform_3D(root, self.L, self.q)
                self.n_leaves = 8 ** self.L
        else:
            self.bool_uniform = False
            self.n_leaves = len(get_all_leaves(root))
            if self.bool_2D:
                self.interior_points = g2.compute_interior_Chebyshev_points_adaptive_2D(root, self.p)
                self.boundary_points = g2.compute_boundary_Gauss_points_adaptive_2D(root, self.q)
            else:
                from . import _grid_creation_3D as g3
                self.interior_points = g3.compute_interior_Chebyshev_points_adaptive_3D(root, self.p)
                self.boundary_points = g3.compute_boundary_Gauss_points_adaptive_3D(root, self.q)

    def leaf_bounds(self) -> np.ndarray:
        """(n_leaves, 2d) leaf boxes (min, max per axis) in leaf order."""
        if self.bool_uniform:
            if self.bool_2D:
                return g2.uniform_leaf_bounds_2D(self.root.bounds, self.L)
            from . import _grid_creation_3D as g3
            return g3.uniform_leaf_bounds_3D(self.root.bounds, self.L)
        from ._interpolation import _leaf_bounds
        return _leaf_bounds(get_all_leaves(self.root))

    def interp_to_interior_points(self, values, sample_points_x, sample_points_y, sample_points_z=None,
                                  host_device="cpu"):
        """Values on the HPS grid (n_leaves, p^d) of the interpolant of
        ``values`` (n_x, n_y) or (n_x, n_y, n_z) given on
        meshgrid(sample_points_x, sample_points_y[, sample_points_z],
        indexing='ij') (src/jaxhps/_domain.py:99-206)."""
        from . import _interpolation as ip
        n = [np.shape(sample_points_x)[0], np.shape(sample_points_y)[0]]
        if self.bool_2D:
            if sample_points_z is not None:
                raise ValueError("sample_points_z is only for 3D domains")
        else:
            if sample_points_z is None:
                raise ValueError("3D domains need sample_points_z")
            n.append(np.shape(sample_points_z)[0])
        if tuple(values.shape) != tuple(n):
            raise ValueError(f"values have shape {tuple(values.shape)}, expected {tuple(n)}")
        if self.bool_2D:
            return ip.interp_to_hps_2D(self.leaf_bounds(), values, self.p, sample_points_x, sample_points_y,
                                       host_device=host_device)
        return ip.interp_to_hps_3D(self.leaf_bounds(), values, self.p, sample_points_x, sample_points_y,
                                   sample_points_z, host_device=host_device)

    def interp_to_boundary_points(self, sample_points, sample_values, sample_f):
        """Not implemented in the reference either (src/jaxhps/_domain.py:208-216)."""
        raise NotImplementedError("interp_to_boundary_points is not implemented yet.")

    def interp_from_interior_points(self, samples, eval_points_x, eval_points_y, eval_points_z=None,
                                    host_device="cpu"):
        """(values on the rectangular grid, target points) of the HPS
        function ``samples`` (n_leaves, p^d[, n_src]) (src/jaxhps/_domain.py
        :218-294)."""
        from . import _interpolation as ip
        if self.bool_2D and eval_points_z is not None:
            raise ValueError("eval_points_z is only for 3D domains")
        if not self.bool_2D and eval_points_z is None:
            raise ValueError("3D domains need eval_points_z")
        n_leaves, n_per_leaf = self.interior_points.shape[:2]
        if tuple(samples.shape[:2]) != (n_leaves, n_per_leaf):
            raise ValueError(f"samples have shape {tuple(samples.shape)}, expected ({n_leaves}, {n_per_leaf}, ...)")
        if self.bool_2D:
            return ip.interp_from_hps_2D(self.leaf_bounds(), self.p, samples, eval_points_x, eval_points_y,
                                         host_device=host_device)
        return ip.interp_from_hps_3D(self.leaf_bounds(), self.p, samples, eval_points_x, eval_points_y,
                                     eval_points_z, host_device=host_device)

    def get_adaptive_boundary_data_lst(self, f: Callable) -> List[np.ndarray]:
        """Boundary data split per side (2D: S, E, N, W) or face (3D: -x, +x,
        -y, +y, -z, +z) as in src/jaxhps/_domain.py:296-365."""
        b = self.boundary_points
        r = self.root
        if self.bool_2D:
            masks = [b[:, 1] == r.ymin, b[:, 0] == r.xmax, b[:, 1] == r.ymax, b[:, 0] == r.xmin]
        else:
            masks = [b[:, 0] == r.xmin, b[:, 0] == r.xmax, b[:, 1] == r.ymin, b[:, 1] == r.ymax,
                     b[:, 2] == r.zmin, b[:, 2] == r.zmax]
        return [f(b[m]) for m in masks]

    @classmethod
    def from_adaptive_discretization(cls, p: int, q: int, root, f, tol: float, use_level_restriction: bool = True,
                                     use_l_2_norm: bool = False, proposer=None) -> "Domain":
        """Adaptive refinement of ``root`` until every leaf resolves ``f``
        to ``tol`` (src/jaxhps/_domain.py:367-434).  ``proposer`` is an
        optional learned refinement proposal (jaxhps_gb300.refinement_mlp);
        the interpolation criterion still decides every accepted leaf."""
        fs = f if isinstance(f, list) else [f]
        if isinstance(root, DiscretizationNode2D):
            from ._adaptive_discretization_2D import generate_adaptive_mesh_level_restriction_2D as gen
        else:
            from ._adaptive_discretization_3D import generate_adaptive_mesh_level_restriction as gen
        for fn in fs:
            kw = dict(root=root, f_fn=fn, tol=tol, p=p, q=q, restrict_bool=use_level_restriction,
                      l2_norm=use_l_2_norm)
            if proposer is not None:
                kw["proposer"] = proposer
            gen(**kw)
        return cls(p=p, q=q, root=root)

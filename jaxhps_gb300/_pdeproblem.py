"""``PDEProblem`` (API mirror of src/jaxhps/_pdeproblem.py:25-505).

Stores the coefficient arrays (each (n_leaves, p^d) on the leaf points), the
source, the ItI flag and eta, the precomputed dense operators, and the
solver state filled in by ``build_solver``: ``Y, v, S_lst, g_tilde_lst,
D_inv_lst, BD_inv_lst, Phi``.  Unlike the reference, the solver state stays
resident in device memory (torch CUDA tensors).
"""

from __future__ import annotations

from typing import List, Tuple

import numpy as np

from ._discretization_tree import DiscretizationNode3D, get_all_leaves
from ._domain import Domain
from . import _precompute_operators_2D as op2

COEFF_NAMES_2D = ("D_xx", "D_xy", "D_yy", "D_x", "D_y", "I")
COEFF_NAMES_3D = ("D_xx", "D_xy", "D_yy", "D_xz", "D_yz", "D_zz", "D_x", "D_y", "D_z", "I")


def _to_numpy(a):
    """Inputs are kept as given (NumPy arrays or torch tensors, possibly in
    pinned host memory); lists are converted to NumPy."""
    if a is None or hasattr(a, "shape"):
        return a
    return np.asarray(a)


class PDEProblem:
    def __init__(self, domain: Domain, source=None, D_xx_coefficients=None, D_xy_coefficients=None,
                 D_xz_coefficients=None, D_yy_coefficients=None, D_yz_coefficients=None,
                 D_zz_coefficients=None, D_x_coefficients=None, D_y_coefficients=None, D_z_coefficients=None,
                 I_coefficients=None, use_ItI: bool = False, eta: float | None = None):
        self.domain = domain
        bool_2D = not isinstance(domain.root, DiscretizationNode3D)
        if not bool_2D:
            if use_ItI:
                raise NotImplementedError("ItI merges are not supported for 3D problems.")
        else:
            for c in (D_xz_coefficients, D_yz_coefficients, D_zz_coefficients, D_z_coefficients):
                if c is not None:
                    raise ValueError("z coefficients can not be set for 2D problems.")
        if use_ItI and eta is None:
            raise ValueError("eta must be specified when using ItI merges.")
        if use_ItI and not domain.bool_uniform:
            raise ValueError("ItI merges are only supported for uniform 2D problems.")
        if source is None and (not bool_2D or not domain.bool_uniform):
            raise ValueError("Source must be specified for non-uniform or 3D problems.")

        coeffs = dict(D_xx=D_xx_coefficients, D_xy=D_xy_coefficients, D_xz=D_xz_coefficients,
                      D_yy=D_yy_coefficients, D_yz=D_yz_coefficients, D_zz=D_zz_coefficients,
                      D_x=D_x_coefficients, D_y=D_y_coefficients, D_z=D_z_coefficients, I=I_coefficients)
        check_input_shapes(domain.interior_points[..., 0].shape, coeffs)
        for k, v in coeffs.items():
            setattr(self, f"{k}_coefficients", _to_numpy(v))
        self.source = _to_numpy(source)
        self.use_ItI = bool(use_ItI)
        self.eta = eta

        if domain.bool_uniform:
            half_side_len = (domain.root.xmax - domain.root.xmin) / (2 ** (domain.L + 1))
        else:
            half_side_len = 1.0
            self.sidelens = np.array([l.xmax - l.xmin for l in get_all_leaves(domain.root)])

        p, q = domain.p, domain.q
        if bool_2D:
            self.D_x, self.D_y, self.D_xx, self.D_yy, self.D_xy = op2.precompute_diff_operators_2D(p, half_side_len)
            if not use_ItI:
                self.P = op2.precompute_P_2D_DtN(p, q)
                self.Q = op2.precompute_Q_2D_DtN(p, q, self.D_x, self.D_y)
            else:
                self.P = op2.precompute_P_2D_ItI(p, q)
                N_tilde = op2.precompute_N_tilde_matrix_2D(self.D_x, self.D_y, p)
                self.G = op2.precompute_G_2D_ItI(N_tilde, self.eta)
                N = op2.precompute_N_matrix_2D(self.D_x, self.D_y, p)
                self.QH = op2.precompute_QH_2D_ItI(N, p, q, self.eta)
            if not domain.bool_uniform:
                self.L_2f1, self.L_1f2 = op2.precompute_projection_ops_2D(q)
        else:
            from . import _precompute_operators_3D as op3
            (self.D_x, self.D_y, self.D_z, self.D_xx, self.D_yy, self.D_zz, self.D_xy, self.D_xz,
             self.D_yz) = op3.precompute_diff_operators_3D(p, half_side_len)
            self.P = op3.precompute_P_3D_DtN(p, q)
            self.Q = op3.precompute_Q_3D_DtN(p, q, self.D_x, self.D_y, self.D_z)
            if not domain.bool_uniform:
                self.L_4f1, self.L_1f4 = op3.precompute_projection_ops_3D(q)

        self.reset()

    # ------------------------------------------------------------------
    def reset(self) -> None:
        """Drops the stored solution operators."""
        self.Y = None
        self.v = None
        self.S_lst: List = []
        self.g_tilde_lst: List = []
        self.D_inv_lst: List = []
        self.BD_inv_lst: List = []
        self._D_inv_int: List = []
        self._BD_inv_int: List = []
        self.Phi = None
        self._state = None

    def update_coefficients(self, source=None, D_xx_coefficients=None, D_xy_coefficients=None,
                            D_xz_coefficients=None, D_yy_coefficients=None, D_yz_coefficients=None,
                            D_zz_coefficients=None, D_x_coefficients=None, D_y_coefficients=None,
                            D_z_coefficients=None, I_coefficients=None) -> None:
        """Replaces the given coefficients (and source) and resets the solver
        state (src/jaxhps/_pdeproblem.py:249-333)."""
        self.reset()
        coeffs = dict(D_xx=D_xx_coefficients, D_xy=D_xy_coefficients, D_xz=D_xz_coefficients,
                      D_yy=D_yy_coefficients, D_yz=D_yz_coefficients, D_zz=D_zz_coefficients,
                      D_x=D_x_coefficients, D_y=D_y_coefficients, D_z=D_z_coefficients, I=I_coefficients)
        check_input_shapes(self.domain.interior_points[..., 0].shape, coeffs)
        if source is not None:
            self.source = _to_numpy(source)
        for k, v in coeffs.items():
            if v is not None:
                setattr(self, f"{k}_coefficients", _to_numpy(v))

    # ------------------------------------------------------------------
    def active_coefficients(self) -> Tuple[list, list]:
        """(coefficient arrays, operator matrices) of the non-None terms, in
        the reference's stacking order (local_solve/_uniform_2D_DtN.py:59-68)."""
        names = COEFF_NAMES_2D if self.domain.bool_2D else COEFF_NAMES_3D
        cs, ops = [], []
        n = self.domain.p ** (2 if self.domain.bool_2D else 3)
        for name in names:
            c = getattr(self, f"{name}_coefficients")
            if c is None:
                continue
            cs.append(c)
            ops.append(np.eye(n) if name == "I" else getattr(self, name))
        return cs, ops


def check_input_shapes(expected_shape, coeffs: dict) -> None:
    for name, arr in coeffs.items():
        if arr is not None and tuple(arr.shape) != tuple(expected_shape):
            raise ValueError(f"{name}_coefficients has shape {tuple(arr.shape)} but should have shape "
                             f"{tuple(expected_shape)} to match the Domain's interior points.")

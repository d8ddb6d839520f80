"""``build_solver`` (API mirror of src/jaxhps/_build_solver.py:38-174).

Runs the leaf stage and the merge stage on the GPU and stores the solution
operators on the ``PDEProblem``.  Extra keyword ``precision``:

* ``"float64"`` (default) - every stage in FP64, the reference's arithmetic.
* ``"float32"``          - every stage in FP32 (no refinement; for study).
* ``"mixed"``            - FP32 build; ``solve`` then refines the FP32
  solution against FP64 residuals of the discrete HPS system until the
  requested tolerance (see ``_refinement.py``).
"""

from __future__ import annotations

import torch

from . import _native as nat
from . import _phases as phases
from . import _stages as st
from ._discretization_tree import DiscretizationNode2D

_PREC = {"float64": torch.float64, "float32": torch.float32, "mixed": torch.float32}


def build_solver(pde_problem, return_top_T: bool = False, compute_device=None, host_device=None,
                 precision: str = "float64", **refine_kw):
    """Builds the solver operators (see the module docstring).  After the
    build, the status words of every batched inverse and the tensor-core
    GEMM's timeout flag are checked (one device sync): a singular leaf or
    merge matrix raises SingularPivotError, a bounded device wait that ran
    out raises DeviceWaitTimeout (both from ``_native``)."""
    if precision not in _PREC:
        raise ValueError(f"precision must be one of {sorted(_PREC)}")
    pde_problem._leaf_info = None
    out = _build(pde_problem, return_top_T, compute_device, precision, **refine_kw)
    st.check_infos([pde_problem._leaf_info], "leaf inverse")
    nat.raise_on_tc_timeout("build_solver")
    return out


@phases.ranged("build_solver")
def _build(pde_problem, return_top_T, compute_device, precision, **refine_kw):
    dom = pde_problem.domain
    if precision == "mixed":
        if pde_problem.use_ItI:
            from ._refinement_iti import build_mixed_iti
            return build_mixed_iti(pde_problem, return_top_T=return_top_T, device=compute_device, **refine_kw)
        if dom.bool_uniform and not dom.bool_2D and not pde_problem.use_ItI:
            from ._refinement_dense import build_mixed_dense
            return build_mixed_dense(pde_problem, return_top_T=return_top_T, device=compute_device, **refine_kw)
        from ._refinement import build_mixed
        return build_mixed(pde_problem, return_top_T=return_top_T, device=compute_device, **refine_kw)
    dtype = _PREC[precision]
    if pde_problem.source is None:
        if not dom.bool_uniform or not isinstance(dom.root, DiscretizationNode2D):
            raise ValueError("Build stage for problems without source terms is only implemented for 2D uniform "
                             "problems.")
        from ._nosource import nosource_build_solver
        return nosource_build_solver(pde_problem, return_top_T=return_top_T, device=compute_device, dtype=dtype)
    if not dom.bool_uniform:
        from ._adaptive import adaptive_build_solver
        return adaptive_build_solver(pde_problem, return_top_T=return_top_T, device=compute_device, dtype=dtype)

    pde_problem._precision = precision
    if pde_problem.use_ItI:
        from . import _iti
        Y, T, v, h = st.local_solve_stage_uniform_2D_ItI(pde_problem, device=compute_device,
                                                         dtype=st.REAL_TO_COMPLEX[dtype])
        pde_problem.Y, pde_problem.v = Y, v
        out = _iti.merge_stage_uniform_2D_ItI(T, h, l=dom.L, device=compute_device, return_T=return_top_T)
    elif dom.bool_2D:
        Y, T, v, h = st.local_solve_stage_uniform_2D_DtN(pde_problem, device=compute_device, dtype=dtype)
        pde_problem.Y, pde_problem.v = Y, v
        out = st.merge_stage_uniform_2D_DtN(T, h, l=dom.L, device=compute_device, return_T=return_top_T)
    else:
        from . import _stages_3D as st3
        Y, T, v, h = st.local_solve_stage_uniform_3D_DtN(pde_problem, device=compute_device, dtype=dtype)
        pde_problem.Y, pde_problem.v = Y, v
        out = st3.merge_stage_uniform_3D_DtN(T, h, l=dom.L, device=compute_device, return_T=return_top_T)
    pde_problem.S_lst, pde_problem.g_tilde_lst = out[0], out[1]
    if return_top_T:
        return out[2]
    return None

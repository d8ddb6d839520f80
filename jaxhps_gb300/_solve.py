"""``solve`` (API mirror of src/jaxhps/_solve.py:18-151).

Propagates boundary data down the merge tree on the GPU and returns the
leaf solutions, shape (n_leaves, p^d) or (n_leaves, p^d, nsrc), on
``host_device`` ("cpu" by default, as in the reference; pass a CUDA device
or None to keep the result in device memory).  ``out``, a tensor of the
result's shape and dtype (for example a page-locked CPU buffer that the
caller reuses), receives the result instead, and is returned; it takes
precedence over ``host_device``.  After a mixed-precision DtN build a
page-locked, contiguous ``out`` is written by the solution's assembly kernel
itself through the buffer's device mapping (no device-side result, no
separate copy).  No counterpart in the reference.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from . import _phases as phases
from . import _stages as st


def solve(pde_problem, boundary_data, source=None, compute_device=None, host_device="cpu", out=None, **refine_kw):
    if out is not None:
        state = getattr(pde_problem, "_state", None)
        if (state is not None and getattr(state, "mixed", False) and not getattr(state, "iti", False)
                and not getattr(state, "dense", False)):
            # the refined DtN solve writes a page-locked `out` directly
            refine_kw = dict(refine_kw, out=out)
        u = _solve(pde_problem, boundary_data, source, compute_device, None, **refine_kw)
        res = out if u is out else st._to_host(u, None, out=out)
    else:
        res = _solve(pde_problem, boundary_data, source, compute_device, host_device, **refine_kw)
    phases.mark("result_d2h")
    nat.raise_on_tc_timeout("solve")
    return res


@phases.ranged("solve")
def _solve(pde_problem, boundary_data, source, compute_device, host_device, **refine_kw):
    dom = pde_problem.domain
    state = getattr(pde_problem, "_state", None)
    if state is not None and getattr(state, "iti", False):
        from ._refinement_iti import solve_mixed_iti
        return solve_mixed_iti(pde_problem, boundary_data, source=source, host_device=host_device, **refine_kw)
    if state is not None and getattr(state, "dense", False):
        from ._refinement_dense import solve_mixed_dense
        return solve_mixed_dense(pde_problem, boundary_data, source=source, host_device=host_device, **refine_kw)
    if state is not None and getattr(state, "mixed", False):
        from ._refinement import solve_mixed
        return solve_mixed(pde_problem, boundary_data, source=source, host_device=host_device, **refine_kw)
    if source is not None:
        if not dom.bool_2D or not dom.bool_uniform:
            raise ValueError("Source can only be specified for 2D uniform problems. For other problems, the source "
                             "must be specified at the time the solver is built.")
        from ._nosource import up_then_down_pass
        return up_then_down_pass(pde_problem, boundary_data, source, device=compute_device, host_device=host_device)
    if not dom.bool_uniform:
        if not isinstance(boundary_data, list):
            raise ValueError("For adaptive solves, boundary data needs to be a list. Try using the "
                             "Domain.get_adaptive_boundary_data_lst() utility.")
        from ._adaptive import adaptive_solve
        return adaptive_solve(pde_problem, boundary_data, device=compute_device, host_device=host_device)
    if isinstance(boundary_data, list):
        if boundary_data and isinstance(boundary_data[0], torch.Tensor):
            boundary_data = torch.cat(boundary_data)
        else:
            boundary_data = np.concatenate([np.asarray(b) for b in boundary_data])
    if pde_problem.use_ItI:
        from . import _iti
        return _iti.down_pass_uniform_2D_ItI(boundary_data, pde_problem.S_lst, pde_problem.g_tilde_lst,
                                             pde_problem.Y, pde_problem.v, device=compute_device,
                                             host_device=host_device)
    if dom.bool_2D:
        return st.down_pass_uniform_2D_DtN(boundary_data, pde_problem.S_lst, pde_problem.g_tilde_lst, pde_problem.Y,
                                           pde_problem.v, device=compute_device, host_device=host_device)
    from . import _stages_3D as st3
    return st3.down_pass_uniform_3D_DtN(boundary_data, pde_problem.S_lst, pde_problem.g_tilde_lst, pde_problem.Y,
                                        pde_problem.v, device=compute_device, host_device=host_device)

"""Save and load the built operator set of a uniform-grid ``PDEProblem``.

``save_solver(pde_problem, path)`` writes what ``build_solver`` left on the
problem (the leaf ``Y``, ``v``, the merge levels' ``S``, ``g_tilde``,
``D_inv``, ``BD_inv``, the no-source up-pass operators and, after a mixed
build, the refinement state with its FP32 operators, coefficients, source
and index tables) as one file of raw tensors plus a manifest of the domain
it was built on.  ``load_solver(pde_problem, path)`` puts that set back on
a problem over the same domain, on the given device, after which ``solve``
runs without a build.  A manifest that does not match the problem's domain
(dimension, p, q, L, root bounds, ItI and eta) raises ValueError.  The file
is a torch pickle (the refinement state is a dataclass): load only files
written by a process you trust.

The reference keeps its solver state on the ``PDEProblem`` object only
(src/jaxhps/_pdeproblem.py:219-234) and has no save/load; its examples save
results with ``scipy.io.savemat``.  Adaptive trees keep their operators on
the tree's nodes and are not covered here.
"""

from __future__ import annotations

import numpy as np
import torch

FORMAT = "jaxhps_gb300.solver/1"

# attributes that build_solver sets (uniform domains), in every precision
_BUILT = ("Y", "v", "S_lst", "g_tilde_lst", "D_inv_lst", "BD_inv_lst", "_D_inv_int", "_BD_inv_int", "Phi",
          "_state", "_precision", "_leaf_info")


def _signature(pde_problem) -> dict:
    dom = pde_problem.domain
    return {
        "dim": 2 if dom.bool_2D else 3,
        "p": int(dom.p),
        "q": int(dom.q),
        "L": int(dom.L),
        "bounds": [float(b) for b in np.asarray(dom.root.bounds, dtype=np.float64).ravel()],
        "use_ItI": bool(pde_problem.use_ItI),
        "eta": None if pde_problem.eta is None else complex(pde_problem.eta),
        "n_leaves": int(dom.n_leaves),
    }


def _check_uniform(pde_problem) -> None:
    if not pde_problem.domain.bool_uniform:
        raise NotImplementedError("save/load of the operator set is implemented for uniform domains; adaptive "
                                  "trees keep their operators on the tree's nodes")


def save_solver(pde_problem, path) -> None:
    """Writes the built operator set of ``pde_problem`` to ``path``."""
    _check_uniform(pde_problem)
    if pde_problem.S_lst is None or (len(pde_problem.S_lst) == 0 and pde_problem.Y is None):
        raise ValueError("nothing to save: build_solver has not run on this problem")
    state = {name: getattr(pde_problem, name, None) for name in _BUILT}
    torch.save({"format": FORMAT, "signature": _signature(pde_problem), "state": state}, path)


def load_solver(pde_problem, path, device=None) -> None:
    """Restores an operator set written by ``save_solver`` onto ``pde_problem``
    (tensors on ``device``, default the current CUDA device)."""
    _check_uniform(pde_problem)
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else "cpu"
    blob = torch.load(path, map_location=device, weights_only=False)
    if not isinstance(blob, dict) or blob.get("format") != FORMAT:
        raise ValueError(f"{path}: not an operator set written by save_solver")
    want, got = _signature(pde_problem), blob["signature"]
    if want != got:
        diff = {k: (got.get(k), want[k]) for k in want if got.get(k) != want[k]}
        raise ValueError(f"{path}: built for another domain (saved, this problem): {diff}")
    pde_problem.reset()
    for name, value in blob["state"].items():
        setattr(pde_problem, name, value)

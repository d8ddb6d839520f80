"""Failures the product path must report instead of returning bad numbers.

* Iterative refinement that runs out of steps raises RefinementNotConverged
  (the reference has no refinement; its solve either succeeds or raises
  ValueError on bad input, _solve.py:53-55).
* A singular leaf matrix (all coefficients zero on a leaf) is caught from
  the batched inverse's status words and raises SingularPivotError.
* A bounded device wait that runs out (the multi-CTA inverse panel's grid
  barrier, made to give up by a poll limit of 0) marks its matrix with
  info = -1 and the inverse finishes without a hang or a fault; the check
  raises DeviceWaitTimeout, and the next call, with the limit restored, is
  correct.  This runs in a child process because the panel kind (cluster or
  cooperative grid) is fixed per process by HPS_CLUSTER_PANELS.
"""

import os
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300 import _native as nat
from jaxhps_gb300 import _stages as st

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def _poisson(L=2, p=8, q=6, zero_leaf=None):
    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=root, L=L)
    x = dom.interior_points
    c = 1.0 + 0.5 * np.exp(-((x[..., 0] - 0.2) ** 2 + x[..., 1] ** 2) / 0.1)
    ones = np.ones_like(c)
    f = np.sin(x[..., 0]) * np.cos(2 * x[..., 1])
    if zero_leaf is not None:
        ones = ones.copy()
        ones[zero_leaf] = 0.0
        c = c.copy()
        c[zero_leaf] = 0.0
    pde = hps.PDEProblem(dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c)
    g = dom.boundary_points[:, 0] ** 2 - dom.boundary_points[:, 1] ** 2
    return pde, g


def test_refinement_out_of_steps_raises(cuda):
    pde, g = _poisson()
    hps.build_solver(pde, precision="mixed")
    with pytest.raises(nat.RefinementNotConverged):
        hps.solve(pde, g, max_iters=1)
    u = hps.solve(pde, g)   # the same build still solves with the default budget
    pde64, _ = _poisson()
    hps.build_solver(pde64)
    u64 = hps.solve(pde64, g)
    assert np.abs(np.asarray(u) - np.asarray(u64)).max() <= 1e-10 * np.abs(np.asarray(u64)).max()


@pytest.mark.parametrize("precision", ["float64", "mixed"])
def test_singular_leaf_raises(cuda, precision):
    pde, _ = _poisson(zero_leaf=5)
    with pytest.raises(nat.SingularPivotError):
        hps.build_solver(pde, precision=precision)


def test_check_infos_reports_each_kind(cuda):
    ok = torch.zeros(4, dtype=torch.int32, device=cuda)
    st.check_infos([ok])
    with pytest.raises(nat.SingularPivotError, match="matrix 2"):
        st.check_infos([ok, torch.tensor([0, 0, 7], dtype=torch.int32, device=cuda)])
    with pytest.raises(nat.DeviceWaitTimeout):
        st.check_infos([torch.tensor([0, -1], dtype=torch.int32, device=cuda)])


def test_tc_status_reset(cuda):
    lib = nat.load_library()
    lib.hps_gemm_tc_status_reset()
    assert lib.hps_gemm_tc_status() == 0
    assert lib.hps_gemm_tc_status_reset() == 0
    nat.raise_on_tc_timeout("test")


def test_spin_limit_setter_round_trip(cuda):
    p0, t0 = nat.set_spin_limits(-1, -1)
    assert p0 > 0 and t0 > 0
    p1, t1 = nat.set_spin_limits(12345, 10)    # tc limit is held at its floor
    assert (p1, t1) == (p0, t0)
    p2, t2 = nat.set_spin_limits(p0, t0)
    assert p2 == 12345 and t2 == 1 << 20


CHILD = textwrap.dedent(
    """
    import sys
    import numpy as np
    import torch
    sys.path.insert(0, sys.argv[1])
    from jaxhps_gb300 import _native as nat, _stages as st
    nat.load_library()
    torch.cuda.set_device(0)
    n = 512
    rng = np.random.default_rng(5)
    A = rng.standard_normal((1, n, n)) + 2 * np.sqrt(n) * np.eye(n)
    At = torch.as_tensor(A, device="cuda")
    prev, _ = nat.set_spin_limits(0, -1)
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    nat.inverse(At, info=info)
    torch.cuda.synchronize()
    assert int(info.item()) == -1, int(info.item())
    try:
        st.check_infos([info])
        raise SystemExit("no DeviceWaitTimeout")
    except nat.DeviceWaitTimeout:
        pass
    nat.set_spin_limits(prev, -1)
    info.zero_()
    X = nat.inverse(At, info=info)
    torch.cuda.synchronize()
    assert int(info.item()) == 0
    ref = np.linalg.inv(A)
    err = np.abs(X.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err < 1e-12, err
    print("CHILD-OK")
    """
)


def test_panel_barrier_timeout_reports_and_recovers(cuda):
    env = dict(os.environ, HPS_CLUSTER_PANELS="0")
    r = subprocess.run([sys.executable, "-c", CHILD, str(ROOT)], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "CHILD-OK" in r.stdout, r.stdout + r.stderr

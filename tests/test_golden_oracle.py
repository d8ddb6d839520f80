"""Pins the FP64 oracle to the reference's own outputs.

The fixtures under ``tests/golden/`` were written by running the unmodified
reference package (``build_solver``, ``solve``, ``Domain`` and its adaptive
meshing) through ``tests/golden/make_fixtures.py``.  Here the oracle's
restatement runs on the same inputs and must reproduce the reference's grids
exactly, its adaptive trees leaf for leaf, and its operators and solutions
to rounding (relative max error <= 1e-11; both are FP64 with different
factorisations).
"""

import numpy as np
import pytest

from _golden import load, matrix_err, rel, same_points
from oracle import hps_oracle as O

TOL = 1e-11


def _ops_2d(fx):
    ones = np.ones_like(fx["I_coefficients"].real)
    c = {"D_xx": ones, "D_yy": ones, "I": fx["I_coefficients"]}
    if "D_x_coefficients" in fx:
        c["D_x"] = fx["D_x_coefficients"]
    return c



def _check_ops(fx, S_lst, g_lst, T_top, squeeze):
    for i, S in enumerate(S_lst):
        assert matrix_err(fx, f"S_{i}", S) < TOL, i
    # g~ is compared on the scale of all levels together: where the particular
    # solution vanishes on an interface (c1's root interfaces x = 0, y = 0),
    # the values there are discretization error, ~1e-9 of the others.
    scale = max(np.abs(fx[f"g_tilde_{i}"]).max() for i in range(len(g_lst)))
    for i, g in enumerate(g_lst):
        g = np.asarray(g)
        if squeeze:
            g = g[..., 0]
        err = np.abs(g.reshape(fx[f"g_tilde_{i}"].shape) - fx[f"g_tilde_{i}"]).max()
        assert err < TOL * scale, i
    assert matrix_err(fx, "T_top", T_top) < TOL


def test_c1_grids_operators_and_solutions():
    fx = load("c1_dtn2d_L3_p8")
    ref = O.Problem2D((-1.0, 1.0, -1.0, 1.0), 3, 8, 6, _ops_2d(fx), fx["source"]).build()
    assert same_points(ref.points, fx["interior_points"])
    assert same_points(ref.boundary_points, fx["boundary_points"])
    _check_ops(fx, ref.S_lst, ref.g_lst, ref.T_top, squeeze=True)
    assert rel(ref.Y, fx["Y"]) < TOL
    assert rel(ref.v[..., 0], fx["v"]) < TOL
    for k in (0, 1):
        assert rel(ref.solve(fx[f"bdry_{k}"]), fx[f"soln_{k}"]) < TOL
    # the discretization error of the manufactured solution, as the reference got it
    assert np.abs(fx["soln_0"] - fx["u_exact"]).max() < 1e-4


def test_c1_interpolation_to_a_regular_grid():
    fx = load("c1_dtn2d_L3_p8")
    bounds = O.uniform_leaf_bounds_2D((-1.0, 1.0, -1.0, 1.0), 3)
    vals, pts = O.oracle_interp_from_hps(bounds, 8, fx["soln_0"], [fx["interp_x"], fx["interp_y"]])
    assert same_points(pts, fx["interp_pts"])
    assert rel(vals, fx["interp_vals"]) < TOL


def test_multisource_with_first_order_term():
    fx = load("dtn2d_multisrc_L2_p10")
    ref = O.Problem2D((0.0, 1.0, -1.0, 1.0), 2, 10, 8, _ops_2d(fx), fx["source"]).build()
    assert same_points(ref.points, fx["interior_points"])
    _check_ops(fx, ref.S_lst, ref.g_lst, ref.T_top, squeeze=False)
    assert rel(ref.solve(fx["bdry"]), fx["soln"]) < TOL


def test_nosource_build_then_source_solve():
    """The reference's no-source build + up pass gives the solution that a
    build with the source gives (same discrete system)."""
    fx = load("dtn2d_nosource_L2_p8")
    ref = O.Problem2D((-1.0, 1.0, -1.0, 1.0), 2, 8, 6, _ops_2d(fx), fx["source"]).build()
    for i, S in enumerate(ref.S_lst):
        assert rel(S, fx[f"S_{i}"]) < TOL
    assert rel(ref.solve(fx["bdry"][:, 0]), fx["soln"][..., 0]) < TOL


@pytest.mark.parametrize("name,nosource", [("iti2d_L2_p10", False), ("iti2d_nosource_L2_p8", True)])
def test_iti_operators_and_solution(name, nosource):
    fx = load(name)
    L, p, q, eta = int(fx["L"]), int(fx["p"]), int(fx["q"]), float(fx["eta"])
    ref = O.Problem2D((-1.0, 1.0, -1.0, 1.0), L, p, q, _ops_2d(fx), fx["source"], iti=True, eta=eta).build()
    assert same_points(ref.points, fx["interior_points"])
    if not nosource:
        _check_ops(fx, ref.S_lst, ref.g_lst, ref.T_top, squeeze=True)
    assert rel(ref.solve(fx["bdry"]), fx["soln"]) < TOL


def test_3d_operators_and_solutions():
    fx = load("dtn3d_L2_p6")
    ones = np.ones_like(fx["I_coefficients"])
    co = {"D_xx": ones, "D_yy": ones, "D_zz": ones, "I": fx["I_coefficients"]}
    ref = O.Problem3D((-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), 2, 6, 4, co, fx["source"]).build()
    assert same_points(ref.points, fx["interior_points"])
    assert same_points(ref.boundary_points, fx["boundary_points"])
    _check_ops(fx, ref.S_lst, ref.g_lst, ref.T_top, squeeze=True)
    for k in (0, 1):
        assert rel(ref.solve(fx[f"bdry_{k}"]), fx[f"soln_{k}"]) < TOL


def _wave_lap(x, x0, a):
    d = x.shape[-1]
    r = np.sqrt(((x - x0) ** 2).sum(-1))
    s = a * (r - 0.7)
    return -2 * a**2 * s / (1 + s**2) ** 2 + (d - 1) * a / (1 + s**2) / r


def test_adaptive_3d_tree_and_solution():
    fx = load("adaptive3d_p6")
    p, q, tol, a, x0 = int(fx["p"]), int(fx["q"]), float(fx["tol"]), float(fx["a"]), fx["x0"]
    root = O.OctNode((0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    O.oracle_adaptive_mesh_3D(root, lambda x: _wave_lap(x, x0, a), tol, p, q)
    leaves = root.leaves()
    assert np.array_equal(np.array([lf.b for lf in leaves]), fx["leaf_bounds"])
    assert np.array_equal(np.array([lf.depth for lf in leaves]), fx["leaf_depths"])
    pts = O.leaf_points_3D(np.array([lf.b for lf in leaves]), p)
    assert same_points(pts, fx["interior_points"])
    ones = np.ones(pts.shape[:2])
    O.oracle_adaptive_build_3D(root, p, q, {"D_xx": ones, "D_yy": ones, "D_zz": ones}, fx["source"])
    assert matrix_err(fx, "T_top", root.T) < TOL
    bdry = np.concatenate([fx[f"bdry_face_{i}"] for i in range(6)])
    u = O.oracle_adaptive_solve_3D(root, bdry)[..., 0]
    assert rel(u, fx["soln"]) < TOL


def test_adaptive_2d_tree_and_solution():
    fx = load("adaptive2d_p8")
    p, q, tol, a, x0 = int(fx["p"]), int(fx["q"]), float(fx["tol"]), float(fx["a"]), fx["x0"]
    root = O.QuadNode((0.0, 1.0, 0.0, 1.0))
    O.oracle_adaptive_mesh_2D(root, lambda x: _wave_lap(x, x0, a), tol, p)
    leaves = root.leaves()
    assert np.array_equal(np.array([lf.b for lf in leaves]), fx["leaf_bounds"])
    assert np.array_equal(np.array([lf.depth for lf in leaves]), fx["leaf_depths"])
    pts = O.leaf_points_2D(np.array([lf.b for lf in leaves]), p)
    assert same_points(pts, fx["interior_points"])
    ones = np.ones(pts.shape[:2])
    O.oracle_adaptive_build_2D(root, p, q, {"D_xx": ones, "D_yy": ones}, fx["source"])
    assert rel(root.T, fx["T_top"]) < TOL
    bdry = np.concatenate([fx[f"bdry_side_{i}"] for i in range(4)])
    u = O.oracle_adaptive_solve_2D(root, bdry, q)[..., 0]
    assert rel(u, fx["soln"]) < TOL


@pytest.mark.parametrize("name,root", [("c1_dtn2d_L3_p8", (-1.0, 1.0, -1.0, 1.0)),
                                       ("dtn2d_multisrc_L2_p10", (0.0, 1.0, -1.0, 1.0)),
                                       ("iti2d_L2_p10", (-1.0, 1.0, -1.0, 1.0)),
                                       ("dtn3d_L2_p6", (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0))])
def test_package_grids_are_the_references(name, root):
    """The package's host-side grid construction (Domain) gives the
    reference's interior and boundary points bit for bit."""
    import jaxhps_gb300 as hps

    fx = load(name)
    node = hps.DiscretizationNode2D(*root) if len(root) == 4 else hps.DiscretizationNode3D(*root)
    dom = hps.Domain(p=int(fx["p"]), q=int(fx["q"]), root=node, L=int(fx["L"]))
    assert same_points(dom.interior_points, fx["interior_points"])
    assert same_points(dom.boundary_points, fx["boundary_points"])


@pytest.mark.parametrize("name,root", [("c1_dtn2d_L3_p8", (-1.0, 1.0, -1.0, 1.0)),
                                       ("dtn2d_multisrc_L2_p10", (0.0, 1.0, -1.0, 1.0))])
@pytest.mark.parametrize("threads", [1, 3])
def test_level_batched_oracle_is_the_reference(name, root, threads):
    """The level-batched oracle (the CPU baseline and the full-size accuracy
    reference of bench.py) reproduces the reference's operators and solutions."""
    from oracle import hps_oracle_level as OL

    fx = load(name)
    pr = OL.LevelProblem2D(root, int(fx["L"]), int(fx["p"]), int(fx["q"]), _ops_2d(fx), fx["source"],
                           threads=threads).build()
    multi = fx["source"].ndim == 3
    _check_ops(fx, pr.S_lst, pr.g_lst, pr.T_top, squeeze=not multi)
    if multi:
        assert rel(pr.solve(fx["bdry"]), fx["soln"]) < TOL
    else:
        for k in (0, 1):
            assert rel(pr.solve(fx[f"bdry_{k}"]), fx[f"soln_{k}"]) < TOL
    pr.close()

"""The CUDA path against the reference's own outputs (the golden fixtures
under ``tests/golden/``, written by running the unmodified reference package;
see ``tests/golden/make_fixtures.py``).

Inputs are taken from the fixtures; grids, adaptive trees, operators and
solutions come from this package's public API (``Domain``,
``Domain.from_adaptive_discretization``, ``PDEProblem``, ``build_solver``,
``solve``, ``Domain.interp_from_interior_points``), which runs every stage
through the C ABI.

Tolerances: the FP64 path <= 1e-11 relative max error (operators and
solutions); the mixed-precision path (FP32 build + FP64-residual
refinement) <= 1e-10 on the solutions.
"""

import numpy as np
import pytest

import jaxhps_gb300 as hps
from _golden import load, matrix_err, rel, same_points, to_np

pytestmark = pytest.mark.gpu

TOL64 = 1e-11
TOL_MIXED = 1e-10


def _coeffs(fx, dim):
    ones = np.ones(fx["interior_points"].shape[:2])
    kw = dict(D_xx_coefficients=ones, D_yy_coefficients=ones)
    if dim == 3:
        kw["D_zz_coefficients"] = ones
    if "I_coefficients" in fx:
        kw["I_coefficients"] = fx["I_coefficients"]
    if "D_x_coefficients" in fx:
        kw["D_x_coefficients"] = fx["D_x_coefficients"]
    return kw


def _check_ops(fx, pde, T_top):
    n = len(pde.S_lst)
    for i in range(n):
        assert matrix_err(fx, f"S_{i}", pde.S_lst[i]) < TOL64, i
    scale = max(np.abs(fx[f"g_tilde_{i}"]).max() for i in range(n))
    for i in range(n):
        g = to_np(pde.g_tilde_lst[i]).reshape(fx[f"g_tilde_{i}"].shape)
        assert np.abs(g - fx[f"g_tilde_{i}"]).max() < TOL64 * scale, i
    assert matrix_err(fx, "T_top", T_top) < TOL64


def _uniform_2d(fx, root, **kw):
    dom = hps.Domain(p=int(fx["p"]), q=int(fx["q"]), root=hps.DiscretizationNode2D(*root), L=int(fx["L"]))
    assert same_points(dom.interior_points, fx["interior_points"])
    assert same_points(dom.boundary_points, fx["boundary_points"])
    return dom


@pytest.mark.parametrize("precision", ["float64", "mixed"])
def test_c1(cuda, precision):
    fx = load("c1_dtn2d_L3_p8")
    dom = _uniform_2d(fx, (-1.0, 1.0, -1.0, 1.0))
    pde = hps.PDEProblem(dom, source=fx["source"], **_coeffs(fx, 2))
    T_top = hps.build_solver(pde, return_top_T=True, precision=precision)
    tol = TOL64 if precision == "float64" else TOL_MIXED
    if precision == "float64":
        _check_ops(fx, pde, T_top)
        assert rel(pde.Y, fx["Y"]) < TOL64
        assert rel(to_np(pde.v).reshape(fx["v"].shape), fx["v"]) < TOL64
    for k in (0, 1):
        u = hps.solve(pde, fx[f"bdry_{k}"])
        assert rel(u, fx[f"soln_{k}"]) < tol, k
    u0 = hps.solve(pde, fx["bdry_0"])
    vals, pts = dom.interp_from_interior_points(to_np(u0), fx["interp_x"], fx["interp_y"])
    assert same_points(pts, fx["interp_pts"])
    assert rel(vals, fx["interp_vals"]) < tol


@pytest.mark.parametrize("precision", ["float64", "mixed"])
def test_multisource_first_order_term(cuda, precision):
    fx = load("dtn2d_multisrc_L2_p10")
    dom = _uniform_2d(fx, (0.0, 1.0, -1.0, 1.0))
    pde = hps.PDEProblem(dom, source=fx["source"], **_coeffs(fx, 2))
    T_top = hps.build_solver(pde, return_top_T=True, precision=precision)
    if precision == "float64":
        _check_ops(fx, pde, T_top)
    u = hps.solve(pde, fx["bdry"])
    assert rel(u, fx["soln"]) < (TOL64 if precision == "float64" else TOL_MIXED)


def test_dtn_nosource_up_pass(cuda):
    fx = load("dtn2d_nosource_L2_p8")
    dom = _uniform_2d(fx, (-1.0, 1.0, -1.0, 1.0))
    pde = hps.PDEProblem(dom, **_coeffs(fx, 2))
    hps.build_solver(pde)
    for i in range(len(pde.S_lst)):
        assert rel(pde.S_lst[i], fx[f"S_{i}"]) < TOL64
        assert rel(pde.D_inv_lst[i], fx[f"D_inv_{i}"]) < TOL64
        assert rel(pde.BD_inv_lst[i], fx[f"BD_inv_{i}"]) < TOL64
    u = hps.solve(pde, fx["bdry"], source=fx["source"])
    assert rel(to_np(u).reshape(fx["soln"].shape), fx["soln"]) < TOL64


@pytest.mark.parametrize("precision", ["float64", "mixed"])
def test_iti(cuda, precision):
    fx = load("iti2d_L2_p10")
    dom = _uniform_2d(fx, (-1.0, 1.0, -1.0, 1.0))
    pde = hps.PDEProblem(dom, source=fx["source"], use_ItI=True, eta=float(fx["eta"]), **_coeffs(fx, 2))
    T_top = hps.build_solver(pde, return_top_T=True, precision=precision)
    if precision == "float64":
        _check_ops(fx, pde, T_top)
    u = hps.solve(pde, fx["bdry"])
    assert rel(u, fx["soln"]) < (TOL64 if precision == "float64" else TOL_MIXED)


def test_iti_nosource_up_pass(cuda):
    fx = load("iti2d_nosource_L2_p8")
    dom = _uniform_2d(fx, (-1.0, 1.0, -1.0, 1.0))
    pde = hps.PDEProblem(dom, use_ItI=True, eta=float(fx["eta"]), **_coeffs(fx, 2))
    hps.build_solver(pde)
    for i in range(len(pde.S_lst)):
        assert rel(pde.S_lst[i], fx[f"S_{i}"]) < TOL64
        assert rel(pde.D_inv_lst[i], fx[f"D_inv_{i}"]) < TOL64
        assert rel(pde.BD_inv_lst[i], fx[f"BD_inv_{i}"]) < TOL64
    u = hps.solve(pde, fx["bdry"], source=fx["source"])
    assert rel(u, fx["soln"]) < TOL64


@pytest.mark.parametrize("precision", ["float64", "mixed"])
def test_3d(cuda, precision):
    fx = load("dtn3d_L2_p6")
    root = hps.DiscretizationNode3D(-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=int(fx["p"]), q=int(fx["q"]), root=root, L=int(fx["L"]))
    assert same_points(dom.interior_points, fx["interior_points"])
    assert same_points(dom.boundary_points, fx["boundary_points"])
    pde = hps.PDEProblem(dom, source=fx["source"], **_coeffs(fx, 3))
    T_top = hps.build_solver(pde, return_top_T=True, precision=precision)
    if precision == "float64":
        _check_ops(fx, pde, T_top)
    for k in (0, 1):
        u = hps.solve(pde, fx[f"bdry_{k}"])
        assert rel(u, fx[f"soln_{k}"]) < (TOL64 if precision == "float64" else TOL_MIXED), k


def _wave_lap(x, x0, a):
    x = np.asarray(x)
    d = x.shape[-1]
    r = np.sqrt(((x - x0) ** 2).sum(-1))
    s = a * (r - 0.7)
    return -2 * a**2 * s / (1 + s**2) ** 2 + (d - 1) * a / (1 + s**2) / r


def _leaf_arrays(root, dim):
    leaves = hps.get_all_leaves(root)
    if dim == 2:
        b = np.array([[lf.xmin, lf.xmax, lf.ymin, lf.ymax] for lf in leaves])
    else:
        b = np.array([[lf.xmin, lf.xmax, lf.ymin, lf.ymax, lf.zmin, lf.zmax] for lf in leaves])
    return b, np.array([lf.depth for lf in leaves])


def test_adaptive_3d_meshing_build_solve(cuda):
    fx = load("adaptive3d_p6")
    p, q, tol, a, x0 = int(fx["p"]), int(fx["q"]), float(fx["tol"]), float(fx["a"]), fx["x0"]
    root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
    dom = hps.Domain.from_adaptive_discretization(p=p, q=q, root=root, f=lambda x: _wave_lap(x, x0, a), tol=tol)
    b, d = _leaf_arrays(root, 3)
    assert np.array_equal(b, fx["leaf_bounds"]) and np.array_equal(d, fx["leaf_depths"])
    assert same_points(dom.interior_points, fx["interior_points"])
    pde = hps.PDEProblem(dom, source=fx["source"], **_coeffs(fx, 3))
    T_top = hps.build_solver(pde, return_top_T=True)
    assert matrix_err(fx, "T_top", T_top) < TOL64
    u = hps.solve(pde, [fx[f"bdry_face_{i}"] for i in range(6)])
    assert rel(u, fx["soln"]) < TOL64


def test_adaptive_2d_meshing_build_solve(cuda):
    fx = load("adaptive2d_p8")
    p, q, tol, a, x0 = int(fx["p"]), int(fx["q"]), float(fx["tol"]), float(fx["a"]), fx["x0"]
    root = hps.DiscretizationNode2D(0.0, 1.0, 0.0, 1.0)
    dom = hps.Domain.from_adaptive_discretization(p=p, q=q, root=root, f=lambda x: _wave_lap(x, x0, a), tol=tol)
    b, d = _leaf_arrays(root, 2)
    assert np.array_equal(b, fx["leaf_bounds"]) and np.array_equal(d, fx["leaf_depths"])
    assert same_points(dom.interior_points, fx["interior_points"])
    pde = hps.PDEProblem(dom, source=fx["source"], **_coeffs(fx, 2))
    T_top = hps.build_solver(pde, return_top_T=True)
    assert rel(T_top, fx["T_top"]) < TOL64
    u = hps.solve(pde, [fx[f"bdry_side_{i}"] for i in range(4)])
    assert rel(u, fx["soln"]) < TOL64

"""Generate the golden fixtures in this folder by running the UNMODIFIED
reference package (meliao/jaxhps, ``src/jaxhps``) on the CPU.

The container that made the fixtures has no ``jax``; the reference is
imported against the NumPy stand-in for the ``jax`` API subset it uses
(``_jaxshim/jax``: ``jax.numpy`` on NumPy with ``.at[]`` updates, ``vmap`` as
a loop, ``jit`` as the identity, ``lax`` control flow on concrete values).
The reference's own code paths run unchanged: ``Domain`` (uniform and
``from_adaptive_discretization``), ``PDEProblem``, ``build_solver``
(``_build_solver.py:38-174``) and ``solve`` (``_solve.py:18-151``).

Usage (from the repository root, with the reference checked out)::

    python tests/golden/make_fixtures.py /path/to/jaxhps/src

Each case is written as ``tests/golden/<case>.npz`` holding the inputs
(grid points, coefficient arrays, sources, boundary data) and the
reference's outputs (``S_lst``, ``g_tilde_lst``, top ``T``, leaf ``Y``/``v``
where small, and solutions).  The tests read only the ``.npz`` files.
"""

from __future__ import annotations

import sys
import time
import warnings
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PI = np.pi


def _setup(ref_src: str):
    sys.path.insert(0, str(HERE / "_jaxshim"))
    sys.path.insert(0, ref_src)
    warnings.simplefilter("ignore", SyntaxWarning)
    import jax  # noqa: F401  (the stand-in)
    import jax.numpy as jnp
    import jaxhps

    global J
    J = jnp.asarray
    return jaxhps


def _pde(jh, dom, source=None, **kw):
    """PDEProblem with every array argument passed as a jax array, as a
    caller of the reference does."""
    kw = {k: (J(v) if isinstance(v, np.ndarray) else v) for k, v in kw.items()}
    return jh.PDEProblem(domain=dom, source=None if source is None else J(source), **kw)


def _np(x):
    return np.asarray(x).view(np.ndarray).copy()


def bumps(rng, n, dim, lo=-0.8, hi=0.8):
    return rng.uniform(lo, hi, size=(n, dim))


def bump_sum(x, centres, width):
    d2 = ((x[..., None, :] - centres) ** 2).sum(-1)
    return np.exp(-d2 / width**2).sum(-1)


PROBE_SEED = 99
MAX_DENSE = 1 << 20


def probe_matrix(n_cols, n_probe=4):
    """Seeded probe vectors; the tests rebuild them with the same call."""
    return np.random.default_rng(PROBE_SEED).standard_normal((n_cols, n_probe))


def _store_matrix(out, key, M):
    """Matrices above 1 MB are stored as M @ probe and every 16th row."""
    M = _np(M)
    if M.nbytes <= MAX_DENSE:
        out[key] = M
        return
    out[key + "_probe"] = M @ probe_matrix(M.shape[-1])
    out[key + "_rows16"] = M[..., ::16, :]


def _store_ops(out, pde, with_leaf=True):
    for i, S in enumerate(pde.S_lst):
        _store_matrix(out, f"S_{i}", S)
    for i, g in enumerate(pde.g_tilde_lst):
        out[f"g_tilde_{i}"] = _np(g)
    if with_leaf:
        out["Y"] = _np(pde.Y)
        out["v"] = _np(pde.v)


# ---------------------------------------------------------------------------
# Uniform 2D DtN
# ---------------------------------------------------------------------------


def case_c1(jh):
    """The 2D variable-coefficient problem: [-1,1]^2, L=3, p=8, q=6, DtN.
    c = 1 + 0.5 * sum of 4 Gaussian bumps (centres U[-0.8,0.8]^2 from
    default_rng(0), width 0.2); u = sin(pi x) sin(pi y), f = (c - 2 pi^2) u;
    boundary data u|dOmega (= 0) and, as a second solve, x^2 - y^2."""
    rng = np.random.default_rng(0)
    z = bumps(rng, 4, 2)
    root = jh.DiscretizationNode2D(xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0)
    dom = jh.Domain(p=8, q=6, root=root, L=3)
    x = _np(dom.interior_points)
    bp = _np(dom.boundary_points)
    c = 1.0 + 0.5 * bump_sum(x, z, 0.2)
    u = np.sin(PI * x[..., 0]) * np.sin(PI * x[..., 1])
    f = (c - 2 * PI**2) * u
    ones = np.ones_like(c)
    pde = _pde(jh, dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c)
    T = jh.build_solver(pde_problem=pde, return_top_T=True)
    g0 = np.sin(PI * bp[:, 0]) * np.sin(PI * bp[:, 1])
    g1 = bp[:, 0] ** 2 - bp[:, 1] ** 2
    u0 = jh.solve(pde_problem=pde, boundary_data=J(g0))
    u1 = jh.solve(pde_problem=pde, boundary_data=J(g1))
    out = dict(L=3, p=8, q=6, bump_centres=z, interior_points=x, boundary_points=bp, I_coefficients=c, source=f,
               bdry_0=g0, bdry_1=g1, soln_0=_np(u0), soln_1=_np(u1), u_exact=u)
    _store_matrix(out, "T_top", T)
    _store_ops(out, pde)
    # Interpolation of the solution onto a regular grid (Domain.interp_from_interior_points).
    xs = np.linspace(-1.0, 1.0, 13)
    ys = np.linspace(-1.0, 1.0, 11)
    vals, pts = dom.interp_from_interior_points(u0, J(xs), J(ys))
    out.update(interp_x=xs, interp_y=ys, interp_vals=_np(vals), interp_pts=_np(pts))
    return out


def case_dtn_multisrc(jh):
    """2D DtN with a first-order coefficient and three sources:
    [0,1]x[-1,1], L=2, p=10, q=8, c = 1 + 0.5 bump, D_x = 0.3 sin(y)."""
    rng = np.random.default_rng(7)
    root = jh.DiscretizationNode2D(xmin=0.0, xmax=1.0, ymin=-1.0, ymax=1.0)
    dom = jh.Domain(p=10, q=8, root=root, L=2)
    x = _np(dom.interior_points)
    bp = _np(dom.boundary_points)
    c = 1.0 + 0.5 * np.exp(-((x[..., 0] - 0.4) ** 2 + (x[..., 1] + 0.3) ** 2) / 0.1)
    ones = np.ones_like(c)
    bx = 0.3 * np.sin(x[..., 1])
    f = rng.standard_normal(x.shape[:2] + (3,))
    g = np.stack([np.sin(bp[:, 0]) + k * bp[:, 1] ** 2 for k in range(3)], -1)
    pde = _pde(jh, dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c,
                        D_x_coefficients=bx)
    T = jh.build_solver(pde_problem=pde, return_top_T=True)
    u = jh.solve(pde_problem=pde, boundary_data=J(g))
    out = dict(L=2, p=10, q=8, interior_points=x, boundary_points=bp, I_coefficients=c, D_x_coefficients=bx,
               source=f, bdry=g, soln=_np(u))
    _store_matrix(out, "T_top", T)
    _store_ops(out, pde, with_leaf=False)
    return out


def case_dtn_nosource(jh):
    """2D DtN built without a source, then solved with one through the up
    pass (_build_solver.py:261-331, _solve.py:_up_then_down_pass):
    [-1,1]^2, L=2, p=8, q=6."""
    rng = np.random.default_rng(11)
    root = jh.DiscretizationNode2D(xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0)
    dom = jh.Domain(p=8, q=6, root=root, L=2)
    x = _np(dom.interior_points)
    bp = _np(dom.boundary_points)
    c = 2.0 + np.cos(x[..., 0] * x[..., 1])
    ones = np.ones_like(c)
    pde = _pde(jh, dom, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c)
    jh.build_solver(pde_problem=pde)
    f = rng.standard_normal(x.shape[:2])
    # The DtN up pass always adds a source axis (up_pass/_uniform_2D_DtN.py:71-76),
    # so the down pass wants boundary data of shape (n_bdry, 1).
    g = (np.cos(bp[:, 0]) - bp[:, 1])[:, None]
    u = jh.solve(pde_problem=pde, boundary_data=J(g), source=J(f))
    out = dict(L=2, p=8, q=6, interior_points=x, boundary_points=bp, I_coefficients=c, source=f, bdry=g,
               soln=_np(u))
    for i, S in enumerate(pde.S_lst):
        out[f"S_{i}"] = _np(S)
    for i, D in enumerate(pde.D_inv_lst):
        out[f"D_inv_{i}"] = _np(D)
    for i, B in enumerate(pde.BD_inv_lst):
        out[f"BD_inv_{i}"] = _np(B)
    return out


# ---------------------------------------------------------------------------
# Uniform 2D ItI (Helmholtz)
# ---------------------------------------------------------------------------


def case_iti(jh):
    """Helmholtz with ItI maps, scattering-style source: [-1,1]^2, L=2,
    p=10, q=8, k=6, eta=k; q(x) = 0.5 * sum of 3 bumps (default_rng(2),
    width 0.3); I = k^2 (1 + q); f = -k^2 q u_in with u_in a plane wave at
    a seeded angle; boundary incoming impedance data from a second wave."""
    rng = np.random.default_rng(2)
    k = 6.0
    z = bumps(rng, 3, 2)
    theta = rng.uniform(0, 2 * PI)
    root = jh.DiscretizationNode2D(xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0)
    dom = jh.Domain(p=10, q=8, root=root, L=2)
    x = _np(dom.interior_points)
    bp = _np(dom.boundary_points)
    qx = 0.5 * bump_sum(x, z, 0.3)
    ones = np.ones_like(qx)
    Icoef = k**2 * (1.0 + qx)
    uin = np.exp(1j * k * (x[..., 0] * np.cos(theta) + x[..., 1] * np.sin(theta)))
    f = -(k**2) * qx * uin
    pde = _pde(jh, dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=Icoef,
                        use_ItI=True, eta=k)
    T = jh.build_solver(pde_problem=pde, return_top_T=True)
    g = np.exp(1j * (bp[:, 0] - 0.5 * bp[:, 1]))
    u = jh.solve(pde_problem=pde, boundary_data=J(g))
    out = dict(L=2, p=10, q=8, k=k, eta=k, theta=theta, interior_points=x, boundary_points=bp, I_coefficients=Icoef,
               source=f, bdry=g, soln=_np(u))
    _store_matrix(out, "T_top", T)
    _store_ops(out, pde, with_leaf=False)
    return out


def case_iti_nosource(jh):
    """ItI built without a source, then solved with one through the up pass
    (up_pass/_uniform_2D_ItI.py): [-1,1]^2, L=2, p=8, q=6, k=5."""
    rng = np.random.default_rng(5)
    k = 5.0
    root = jh.DiscretizationNode2D(xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0)
    dom = jh.Domain(p=8, q=6, root=root, L=2)
    x = _np(dom.interior_points)
    bp = _np(dom.boundary_points)
    ones = np.ones(x.shape[:2])
    Icoef = k**2 * (1.0 + 0.2 * np.sin(x[..., 0] + 2 * x[..., 1]))
    pde = _pde(jh, dom, D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=Icoef,
                        use_ItI=True, eta=k)
    jh.build_solver(pde_problem=pde)
    f = rng.standard_normal(x.shape[:2]) + 1j * rng.standard_normal(x.shape[:2])
    g = np.exp(1j * bp[:, 0]) * (1 + bp[:, 1])
    u = jh.solve(pde_problem=pde, boundary_data=J(g), source=J(f))
    out = dict(L=2, p=8, q=6, k=k, eta=k, interior_points=x, boundary_points=bp, I_coefficients=Icoef, source=f,
               bdry=g, soln=_np(u))
    for i, S in enumerate(pde.S_lst):
        out[f"S_{i}"] = _np(S)
    for i, D in enumerate(pde.D_inv_lst):
        out[f"D_inv_{i}"] = _np(D)
    for i, B in enumerate(pde.BD_inv_lst):
        out[f"BD_inv_{i}"] = _np(B)
    return out


# ---------------------------------------------------------------------------
# Uniform 3D DtN
# ---------------------------------------------------------------------------


def case_dtn3d(jh):
    """3D variable-coefficient problem: [-1,1]^3, L=2, p=6, q=4, DtN.
    c = 1 + 0.3 * sum of 6 bumps (default_rng(3), width 0.2);
    u = sin(pi x) sin(pi y) sin(pi z), f = (c - 3 pi^2) u; boundary data u
    (= 0) and, as a second solve, x^2 - y^2 + z."""
    rng = np.random.default_rng(3)
    z = bumps(rng, 6, 3)
    root = jh.DiscretizationNode3D(xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0, zmin=-1.0, zmax=1.0)
    dom = jh.Domain(p=6, q=4, root=root, L=2)
    x = _np(dom.interior_points)
    bp = _np(dom.boundary_points)
    c = 1.0 + 0.3 * bump_sum(x, z, 0.2)
    u = np.sin(PI * x[..., 0]) * np.sin(PI * x[..., 1]) * np.sin(PI * x[..., 2])
    f = (c - 3 * PI**2) * u
    ones = np.ones_like(c)
    pde = _pde(jh, dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones,
                        D_zz_coefficients=ones, I_coefficients=c)
    T = jh.build_solver(pde_problem=pde, return_top_T=True)
    g0 = np.sin(PI * bp[:, 0]) * np.sin(PI * bp[:, 1]) * np.sin(PI * bp[:, 2])
    g1 = bp[:, 0] ** 2 - bp[:, 1] ** 2 + bp[:, 2]
    u0 = jh.solve(pde_problem=pde, boundary_data=J(g0))
    u1 = jh.solve(pde_problem=pde, boundary_data=J(g1))
    out = dict(L=2, p=6, q=4, bump_centres=z, interior_points=x, boundary_points=bp, I_coefficients=c, source=f,
               bdry_0=g0, bdry_1=g1, soln_0=_np(u0), soln_1=_np(u1), u_exact=u)
    _store_matrix(out, "T_top", T)
    _store_ops(out, pde, with_leaf=False)
    return out


# ---------------------------------------------------------------------------
# Adaptive meshing + build + solve
# ---------------------------------------------------------------------------


def _tree_arrays(jh, root, dim):
    leaves = jh.get_all_leaves(root)
    if dim == 2:
        b = np.array([[lf.xmin, lf.xmax, lf.ymin, lf.ymax] for lf in leaves])
    else:
        b = np.array([[lf.xmin, lf.xmax, lf.ymin, lf.ymax, lf.zmin, lf.zmax] for lf in leaves])
    d = np.array([lf.depth for lf in leaves])
    return b, d


def wavefront(x, x0, a):
    r = np.sqrt(((x - x0) ** 2).sum(-1))
    return np.arctan(a * (r - 0.7))


def wavefront_lap(x, x0, a):
    """Laplacian of arctan(a (r - 0.7)) in d = x.shape[-1] dimensions."""
    d = x.shape[-1]
    r = np.sqrt(((x - x0) ** 2).sum(-1))
    s = a * (r - 0.7)
    g1 = a / (1 + s**2)
    g2 = -2 * a**2 * s / (1 + s**2) ** 2
    return g2 + (d - 1) * g1 / r


def case_adaptive3d(jh):
    """Adaptive octree meshing (L-infinity criterion, 2:1 balance) of the
    wavefront source f = Laplacian of arctan(10 (|x - x0| - 0.7)),
    x0 = (-0.05,)*3, on [0,1]^3 with p=6, q=4, tol 1e-2; then build and
    solve Laplace u = f with Dirichlet data u on the adaptive tree."""
    x0 = np.array([-0.05, -0.05, -0.05])
    a = 10.0
    root = jh.DiscretizationNode3D(xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0, zmin=0.0, zmax=1.0)

    def f_fn(x):
        return wavefront_lap(np.asarray(x), x0, a)

    dom = jh.Domain.from_adaptive_discretization(p=6, q=4, root=root, f=f_fn, tol=1e-2)
    bounds, depths = _tree_arrays(jh, root, 3)
    x = _np(dom.interior_points)
    ones = np.ones(x.shape[:2])
    f = f_fn(x)
    pde = _pde(jh, dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones,
                        D_zz_coefficients=ones)
    T = jh.build_solver(pde_problem=pde, return_top_T=True)
    bl = dom.get_adaptive_boundary_data_lst(lambda pts: wavefront(np.asarray(pts), x0, a))
    u = jh.solve(pde_problem=pde, boundary_data=[J(b) for b in bl])
    out = dict(p=6, q=4, tol=1e-2, a=a, x0=x0, leaf_bounds=bounds, leaf_depths=depths, interior_points=x,
               source=f, soln=_np(u), u_exact=wavefront(x, x0, a),
               boundary_points=_np(dom.boundary_points))
    _store_matrix(out, "T_top", T)
    for i, b in enumerate(bl):
        out[f"bdry_face_{i}"] = _np(b)
    return out


def case_adaptive2d(jh):
    """Adaptive quadtree meshing (L-infinity, 2:1 balance) of the 2D
    wavefront source (a = 20) on [0,1]^2 with p=8, q=6, tol 1e-4; then
    build and solve on the adaptive tree with Dirichlet data u."""
    x0 = np.array([-0.05, -0.05])
    a = 20.0
    root = jh.DiscretizationNode2D(xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0)

    def f_fn(x):
        return wavefront_lap(np.asarray(x), x0, a)

    dom = jh.Domain.from_adaptive_discretization(p=8, q=6, root=root, f=f_fn, tol=1e-4)
    bounds, depths = _tree_arrays(jh, root, 2)
    x = _np(dom.interior_points)
    ones = np.ones(x.shape[:2])
    f = f_fn(x)
    pde = _pde(jh, dom, source=f, D_xx_coefficients=ones, D_yy_coefficients=ones)
    T = jh.build_solver(pde_problem=pde, return_top_T=True)
    bl = dom.get_adaptive_boundary_data_lst(lambda pts: wavefront(np.asarray(pts), x0, a))
    u = jh.solve(pde_problem=pde, boundary_data=[J(b) for b in bl])
    out = dict(p=8, q=6, tol=1e-4, a=a, x0=x0, leaf_bounds=bounds, leaf_depths=depths, interior_points=x,
               source=f, soln=_np(u), u_exact=wavefront(x, x0, a),
               boundary_points=_np(dom.boundary_points))
    _store_matrix(out, "T_top", T)
    for i, b in enumerate(bl):
        out[f"bdry_side_{i}"] = _np(b)
    return out


CASES = {
    "c1_dtn2d_L3_p8": case_c1,
    "dtn2d_multisrc_L2_p10": case_dtn_multisrc,
    "dtn2d_nosource_L2_p8": case_dtn_nosource,
    "iti2d_L2_p10": case_iti,
    "iti2d_nosource_L2_p8": case_iti_nosource,
    "dtn3d_L2_p6": case_dtn3d,
    "adaptive3d_p6": case_adaptive3d,
    "adaptive2d_p8": case_adaptive2d,
}


def main(argv):
    ref_src = argv[1] if len(argv) > 1 else "/root/reference/src"
    only = set(argv[2:])
    jh = _setup(ref_src)
    for name, fn in CASES.items():
        if only and name not in only:
            continue
        t = time.time()
        out = fn(jh)
        out["generator"] = np.array("meliao/jaxhps src/jaxhps (unmodified) on the NumPy jax stand-in, "
                                    "tests/golden/make_fixtures.py")
        np.savez_compressed(HERE / f"{name}.npz", **out)
        size = (HERE / f"{name}.npz").stat().st_size
        print(f"{name}: {time.time() - t:.1f} s, {size / 1e6:.2f} MB")


if __name__ == "__main__":
    main(sys.argv)

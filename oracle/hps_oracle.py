"""FP64 CPU oracle for the HPS build/solve path (TEST INFRASTRUCTURE ONLY).

This module is a plain NumPy/SciPy restatement of the reference
(meliao/jaxhps) algorithm for the leaf-solve -> merge -> down-pass path.
It exists only to check the CUDA product path: it may be imported by
``tests/``, by ``__graft_entry__.smoke()`` and by ``bench.py``'s CPU
baseline leg, and by nothing else.  The product package never imports it.

Parity pinning: the reference (JAX, un-pinned ``jax>=0.4``) cannot be run in
this environment, and its test-suite stores no golden vectors.  The oracle is
pinned instead against the reference's own analytic known-answer tests
(polynomial data reproduced to 1e-12, ``tests/test_accuracy/*``), which the
CPU test-suite re-runs against this module.  Raw bitwise parity with JAX's
``jnp.linalg.inv`` output is therefore *unpinned*; agreement is to rounding.

Every function cites the reference file:line it restates (paths relative to
the reference project root).  The code is written per-leaf / per-merge with
explicit loops where that keeps the index bookkeeping readable.
"""

from __future__ import annotations

import numpy as np

# ---------------------------------------------------------------------------
# Quadrature  (src/jaxhps/quadrature/_discretization.py, _differentiation.py,
#              _interpolation.py)
# ---------------------------------------------------------------------------


def chebyshev_points(n: int) -> np.ndarray:
    """Chebyshev-Lobatto points on [-1, 1], left end first.

    Restates quadrature/_discretization.py:12-37:
    ``out[i] = cos(pi * (n-1-i)/(n-1))``.
    """
    angles = np.flipud(np.pi * (np.arange(n, dtype=np.float64) / (n - 1)))
    return np.cos(angles)


def gauss_points(n: int) -> np.ndarray:
    """Gauss-Legendre nodes (quadrature/_discretization.py:104-116)."""
    return np.polynomial.legendre.leggauss(n)[0]


def affine_transform(pts: np.ndarray, ab) -> np.ndarray:
    """Map [-1,1] -> [a,b] (quadrature/_discretization.py:89-101)."""
    a, b = ab
    return 0.5 * (b - a) * pts + 0.5 * (a + b)


def differentiation_matrix_1D(x: np.ndarray) -> np.ndarray:
    """Chebyshev spectral differentiation matrix (Trefethen, Spectral Methods
    in MATLAB ch.6), as in quadrature/_differentiation.py:8-47."""
    p = x.shape[0]
    c = np.ones(p)
    c[0] = 2.0
    c[-1] = 2.0
    c[1::2] *= -1.0
    dx = x[:, None] - x[None, :]
    d = np.outer(c, 1.0 / c) / (dx + np.eye(p))
    d = d - np.diag(d.sum(axis=1))
    return d


def barycentric_matrix_1D(from_pts: np.ndarray, to_pts: np.ndarray) -> np.ndarray:
    """Barycentric Lagrange interpolation matrix (to x from).

    Restates quadrature/_interpolation.py:17-114, including the exact-match
    rows that become unit rows.
    """
    n = from_pts.shape[0]
    w = np.ones(n)
    for j in range(n):
        for k in range(n):
            if j != k:
                w[j] *= from_pts[k] - from_pts[j]
    m = np.zeros((to_pts.shape[0], n))
    for i, t in enumerate(to_pts):
        hit = np.nonzero(t == from_pts)[0]
        if hit.size:
            m[i, hit[0]] = 1.0
            continue
        terms = 1.0 / (w * (t - from_pts))
        m[i] = terms / terms.sum()
    return m


# ---------------------------------------------------------------------------
# 2D leaf grid ordering  (src/jaxhps/_grid_creation_2D.py)
# ---------------------------------------------------------------------------


def ext_first_order_2D(n: int) -> np.ndarray:
    """Permutation from meshgrid(x, flipud(y), 'ij') flat order to the
    exterior-first order of _grid_creation_2D.py:203-233.

    Flat index ``j = ix*n + iy`` with ``iy=0`` the north row.  Boundary runs
    counter-clockwise from the SW corner: south (W->E, n points), east
    (S->N, n-1), north (E->W, n-1, ends on the NW corner), west (N->S, n-2);
    then the interior in increasing flat index.
    """
    order = []
    order += [ix * n + (n - 1) for ix in range(n)]               # south
    order += [(n - 1) * n + iy for iy in range(n - 2, -1, -1)]   # east
    order += [ix * n + 0 for ix in range(n - 2, -1, -1)]         # north
    order += [0 * n + iy for iy in range(1, n - 1)]              # west
    seen = set(order)
    order += [j for j in range(n * n) if j not in seen]
    return np.array(order, dtype=np.int64)


def quad_children_bounds(b):
    """SW, SE, NE, NW children (_grid_creation_2D.py:34-46)."""
    xmin, xmax, ymin, ymax = b
    xm = (xmin + xmax) / 2
    ym = (ymin + ymax) / 2
    return [
        (xmin, xm, ymin, ym),
        (xm, xmax, ymin, ym),
        (xm, xmax, ym, ymax),
        (xmin, xm, ym, ymax),
    ]


def uniform_leaf_bounds_2D(root_bounds, L: int) -> np.ndarray:
    """Leaf boxes in the reference's uniform order (_grid_creation_2D.py:18-31,
    repeated SW/SE/NE/NW subdivision flattened level by level)."""
    boxes = [tuple(root_bounds)]
    for _ in range(L):
        nxt = []
        for b in boxes:
            nxt += quad_children_bounds(b)
        boxes = nxt
    return np.array(boxes, dtype=np.float64)


def leaf_points_2D(bounds: np.ndarray, p: int) -> np.ndarray:
    """Chebyshev points of each leaf, exterior first
    (_grid_creation_2D.py:49-68)."""
    c = chebyshev_points(p)
    r = ext_first_order_2D(p)
    out = np.empty((bounds.shape[0], p * p, 2))
    for i, (xmin, xmax, ymin, ymax) in enumerate(bounds):
        xs = affine_transform(c, (xmin, xmax))
        ys = affine_transform(c, (ymin, ymax))
        X, Y = np.meshgrid(xs, np.flipud(ys), indexing="ij")
        pts = np.stack([X.ravel(), Y.ravel()], axis=-1)
        out[i] = pts[r]
    return out


def boundary_gauss_points_2D(root_bounds, L: int, q: int) -> np.ndarray:
    """Root boundary Gauss points: S (x up), E (y up), N (x down), W (y down)
    (_grid_creation_2D.py:76-124)."""
    xmin, xmax, ymin, ymax = root_bounds
    g = gauss_points(q)
    n = 2 ** L
    xb = np.linspace(xmin, xmax, n + 1)
    yb = np.linspace(ymin, ymax, n + 1)
    xg = np.concatenate([affine_transform(g, xb[i:i + 2]) for i in range(n)])
    yg = np.concatenate([affine_transform(g, yb[i:i + 2]) for i in range(n)])
    return np.concatenate([
        np.stack([xg, np.full_like(xg, ymin)], -1),
        np.stack([np.full_like(yg, xmax), yg], -1),
        np.stack([xg[::-1], np.full_like(xg, ymax)], -1),
        np.stack([np.full_like(yg, xmin), yg[::-1]], -1),
    ])


# ---------------------------------------------------------------------------
# 2D operators  (src/jaxhps/_precompute_operators_2D.py)
# ---------------------------------------------------------------------------


def diff_operators_2D(p: int, half_side_len: float):
    """D_x, D_y, D_xx, D_yy, D_xy in exterior-first order
    (_precompute_operators_2D.py:16-44)."""
    r = ext_first_order_2D(p)
    d = differentiation_matrix_1D(chebyshev_points(p)) / half_side_len
    dx = np.kron(d, np.eye(p))[np.ix_(r, r)]
    dy = -np.kron(np.eye(p), d)[np.ix_(r, r)]
    return dx, dy, dx @ dx, dy @ dy, dx @ dy


def P_2D_DtN(p: int, q: int) -> np.ndarray:
    """Gauss (4q) -> Chebyshev boundary (4(p-1)); corners averaged
    (_precompute_operators_2D.py:48-79)."""
    P = barycentric_matrix_1D(gauss_points(q), chebyshev_points(p))
    out = np.zeros((4 * (p - 1), 4 * q))
    out[0:p, 0:q] = P
    out[p - 1:2 * p - 1, q:2 * q] = P
    out[2 * (p - 1):3 * p - 2, 2 * q:3 * q] = P
    out[3 * (p - 1):, 3 * q:] = P[:-1]
    out[0, 3 * q:] = P[-1]
    for r in (0, p - 1, 2 * (p - 1), 3 * (p - 1)):
        out[r] /= 2.0
    return out


def P_2D_ItI(p: int, q: int) -> np.ndarray:
    """kron(I_4, P[:-1]) (_precompute_operators_2D.py:83-99)."""
    P = barycentric_matrix_1D(gauss_points(q), chebyshev_points(p))
    return np.kron(np.eye(4), P[:-1])


def N_matrix_2D(dx, dy, p):
    """Outward normal derivative on the 4p doubled-corner Chebyshev boundary
    (_precompute_operators_2D.py:132-163)."""
    N = np.zeros((4 * p, p * p))
    N[:p] = -dy[:p]
    N[p:2 * p] = dx[p - 1:2 * p - 1]
    N[2 * p:3 * p] = dy[2 * p - 2:3 * p - 2]
    N[3 * p:4 * p - 1] = -dx[3 * p - 3:4 * p - 4]
    N[4 * p - 1] = -dx[0]
    return N


def N_tilde_matrix_2D(dx, dy, p):
    """Normal derivative at the 4(p-1) boundary points
    (_precompute_operators_2D.py:166-192)."""
    N = np.zeros((4 * (p - 1), p * p))
    N[:p - 1] = -dy[:p - 1]
    N[p - 1:2 * (p - 1)] = dx[p - 1:2 * (p - 1)]
    N[2 * (p - 1):3 * (p - 1)] = dy[2 * (p - 1):3 * (p - 1)]
    N[3 * (p - 1):] = -dx[3 * (p - 1):4 * (p - 1)]
    return N


def Q_2D_DtN(p, q, dx, dy):
    """Interior -> outward normal derivative at the 4q Gauss nodes
    (_precompute_operators_2D.py:102-129)."""
    Qi = barycentric_matrix_1D(chebyshev_points(p), gauss_points(q))
    return np.kron(np.eye(4), Qi) @ N_matrix_2D(dx, dy, p)


def QH_2D_ItI(p, q, dx, dy, eta):
    """Outgoing impedance u_n - i eta u at the Gauss nodes
    (_precompute_operators_2D.py:195-240)."""
    H = N_matrix_2D(dx, dy, p).astype(np.complex128)
    I = np.eye(p)
    H[:p, :p] -= 1j * eta * I
    H[p:2 * p, p - 1:2 * p - 1] -= 1j * eta * I
    H[2 * p:3 * p, 2 * p - 2:3 * p - 2] -= 1j * eta * I
    H[3 * p:4 * p - 1, 3 * p - 3:4 * p - 4] -= 1j * eta * np.eye(p - 1)
    H[4 * p - 1, 0] -= 1j * eta
    Qi = barycentric_matrix_1D(chebyshev_points(p), gauss_points(q))
    return np.kron(np.eye(4), Qi) @ H


def G_2D_ItI(dx, dy, p, eta):
    """Incoming impedance u_n + i eta u at the 4(p-1) Chebyshev boundary
    points (_precompute_operators_2D.py:243-265)."""
    G = N_tilde_matrix_2D(dx, dy, p).astype(np.complex128)
    m = G.shape[0]
    G[:m, :m] += 1j * eta * np.eye(m)
    return G


# ---------------------------------------------------------------------------
# Leaf stage  (src/jaxhps/local_solve/_uniform_2D_DtN.py, _uniform_2D_ItI.py)
# ---------------------------------------------------------------------------


def assemble_operator(coeffs: dict, ops: dict, n_leaves: int, n_pts: int):
    """A = sum_k diag(c_k) D_k per leaf (local_solve/_uniform_2D_DtN.py:182-218).

    ``coeffs`` maps operator names to (n_leaves, n_pts) arrays (or None),
    ``ops`` maps the same names to (n_pts, n_pts) matrices.
    """
    dtype = np.result_type(*[c for c in coeffs.values() if c is not None])
    A = np.zeros((n_leaves, n_pts, n_pts), dtype=np.result_type(dtype, np.float64))
    for name, c in coeffs.items():
        if c is None:
            continue
        A += c[:, :, None] * ops[name][None, :, :]
    return A


def leaf_dtn(A: np.ndarray, f: np.ndarray, P: np.ndarray, Q: np.ndarray):
    """Leaf DtN solve for each leaf (local_solve/_uniform_2D_DtN.py:228-273).

    A: (n_leaves, n, n); f: (n_leaves, n, nsrc).  Returns Y, T, v, h.
    """
    n_cb = P.shape[0]
    nl, n, _ = A.shape
    ns = f.shape[-1]
    Y = np.empty((nl, n, P.shape[1]), dtype=A.dtype)
    v = np.zeros((nl, n, ns), dtype=np.result_type(A.dtype, f.dtype))
    for i in range(nl):
        Aii_inv = np.linalg.inv(A[i, n_cb:, n_cb:])
        Aie = A[i, n_cb:, :n_cb]
        L2 = np.vstack([np.eye(n_cb), -Aii_inv @ Aie])
        Y[i] = L2 @ P
        v[i, n_cb:] = Aii_inv @ f[i, n_cb:]
    T = np.einsum("ab,lbc->lac", Q, Y)
    h = np.einsum("ab,lbc->lac", Q, v)
    return Y, T, v, h


def leaf_iti(A: np.ndarray, f: np.ndarray, P: np.ndarray, QH: np.ndarray,
             G: np.ndarray):
    """Leaf ItI solve (local_solve/_uniform_2D_ItI.py:120-186)."""
    n_cb = P.shape[0]
    nl, n, _ = A.shape
    ns = f.shape[-1]
    Y = np.empty((nl, n, P.shape[1]), dtype=np.complex128)
    v = np.empty((nl, n, ns), dtype=np.complex128)
    for i in range(nl):
        B = np.zeros((n, n), dtype=np.complex128)
        B[:n_cb] = G
        B[n_cb:] = A[i, n_cb:]
        Binv = np.linalg.inv(B)
        Y[i] = Binv[:, :n_cb] @ P
        v[i] = Binv[:, n_cb:] @ f[i, n_cb:]
    T = np.einsum("ab,lbc->lac", QH, Y)
    h = np.einsum("ab,lbc->lac", QH, v)
    return Y, T, v, h


# ---------------------------------------------------------------------------
# Quad merge, DtN  (src/jaxhps/merge/_uniform_2D_DtN.py:206-475,
#                   merge/_schur_complement.py:117-237)
# ---------------------------------------------------------------------------


def _quad_side_indices(nc: int):
    """Per-child index lists of merge/_uniform_2D_DtN.py:384-437.

    Returns dict child -> (outer, first_interface, second_interface) with the
    interface labels used by the reference (5: a|b, 6: b|c, 7: c|d, 8: d|a).
    """
    ix = np.arange(4 * nc)
    a = (np.concatenate([ix[-nc:], ix[:nc]]), ix[nc:2 * nc], ix[2 * nc:3 * nc][::-1])
    b = (ix[:2 * nc], ix[2 * nc:3 * nc], ix[3 * nc:][::-1])
    c = (ix[:nc][::-1], ix[nc:3 * nc], ix[3 * nc:])
    d = (ix[:nc], ix[nc:2 * nc][::-1], ix[2 * nc:])
    return a, b, c, d


def _sub(T, i, j):
    return T[np.ix_(i, j)]


def quad_merge_dtn(Ta, Tb, Tc, Td, ha, hb, hc, hd):
    """One DtN quad merge (merge/_uniform_2D_DtN.py:206-348).

    h* have shape (4nc, nsrc).  Returns S, T, h_out, g_tilde with the
    exterior already rolled by -nc (:343-346).
    """
    nc = Ta.shape[0] // 4
    (a1, a5, a8), (b2, b6, b5), (c6, c3, c7), (d8, d7, d4) = _quad_side_indices(nc)
    z_ei = np.zeros((2 * nc, nc))
    z_ie = np.zeros((nc, 2 * nc))
    z_ii = np.zeros((nc, nc))
    B = np.block([
        [_sub(Ta, a1, a5), z_ei, z_ei, _sub(Ta, a1, a8)],
        [_sub(Tb, b2, b5), _sub(Tb, b2, b6), z_ei, z_ei],
        [z_ei, _sub(Tc, c3, c6), _sub(Tc, c3, c7), z_ei],
        [z_ei, z_ei, _sub(Td, d4, d7), _sub(Td, d4, d8)],
    ])
    C = np.block([
        [_sub(Ta, a5, a1), _sub(Tb, b5, b2), z_ie, z_ie],
        [z_ie, _sub(Tb, b6, b2), _sub(Tc, c6, c3), z_ie],
        [z_ie, z_ie, _sub(Tc, c7, c3), _sub(Td, d7, d4)],
        [_sub(Ta, a8, a1), z_ie, z_ie, _sub(Td, d8, d4)],
    ])
    D = np.block([
        [_sub(Ta, a5, a5) + _sub(Tb, b5, b5), _sub(Tb, b5, b6), z_ii, _sub(Ta, a5, a8)],
        [_sub(Tb, b6, b5), _sub(Tb, b6, b6) + _sub(Tc, c6, c6), _sub(Tc, c6, c7), z_ii],
        [z_ii, _sub(Tc, c7, c6), _sub(Tc, c7, c7) + _sub(Td, d7, d7), _sub(Td, d7, d8)],
        [_sub(Ta, a8, a5), z_ii, _sub(Td, d8, d7), _sub(Td, d8, d8) + _sub(Ta, a8, a8)],
    ])
    dh = np.concatenate([ha[a5] + hb[b5], hb[b6] + hc[c6], hc[c7] + hd[d7], hd[d8] + ha[a8]])
    h_ext = np.concatenate([ha[a1], hb[b2], hc[c3], hd[d4]])
    Dinv = np.linalg.inv(D)
    S = -Dinv @ C
    T = B @ S
    A_blocks = [_sub(Ta, a1, a1), _sub(Tb, b2, b2), _sub(Tc, c3, c3), _sub(Td, d4, d4)]
    for k, Ak in enumerate(A_blocks):
        sl = slice(2 * nc * k, 2 * nc * (k + 1))
        T[sl, sl] += Ak
    g_tilde = -Dinv @ dh
    h_out = h_ext + B @ g_tilde
    h_out = np.roll(h_out, -nc, axis=0)
    T = np.roll(np.roll(T, -nc, axis=0), -nc, axis=1)
    S = np.roll(S, -nc, axis=1)
    return S, T, h_out, g_tilde


def quad_merge_iti(Ra, Rb, Rc, Rd, ha, hb, hc, hd):
    """One ItI quad merge (merge/_uniform_2D_ItI.py:182-375 with
    merge/_schur_complement.py:6-41, 78-114, 182-237)."""
    nc = Ra.shape[0] // 4
    (a1, a5, a8), (b2, b6, b5), (c6, c3, c7), (d8, d7, d4) = _quad_side_indices(nc)
    z_ei = np.zeros((2 * nc, nc))
    z_ie = np.zeros((nc, 2 * nc))
    z_ii = np.zeros((nc, nc))
    B = np.block([
        [_sub(Ra, a1, a5), _sub(Ra, a1, a8), z_ei, z_ei, z_ei, z_ei, z_ei, z_ei],
        [z_ei, z_ei, z_ei, z_ei, _sub(Rb, b2, b5), _sub(Rb, b2, b6), z_ei, z_ei],
        [z_ei, z_ei, _sub(Rc, c3, c6), _sub(Rc, c3, c7), z_ei, z_ei, z_ei, z_ei],
        [z_ei, z_ei, z_ei, z_ei, z_ei, z_ei, _sub(Rd, d4, d7), _sub(Rd, d4, d8)],
    ])
    C = np.block([
        [z_ie, _sub(Rb, b5, b2), z_ie, z_ie],
        [z_ie, z_ie, z_ie, _sub(Rd, d8, d4)],
        [z_ie, _sub(Rb, b6, b2), z_ie, z_ie],
        [z_ie, z_ie, z_ie, _sub(Rd, d7, d4)],
        [_sub(Ra, a5, a1), z_ie, z_ie, z_ie],
        [z_ie, z_ie, _sub(Rc, c6, c3), z_ie],
        [z_ie, z_ie, _sub(Rc, c7, c3), z_ie],
        [_sub(Ra, a8, a1), z_ie, z_ie, z_ie],
    ])
    D12 = np.block([
        [_sub(Rb, b5, b5), _sub(Rb, b5, b6), z_ii, z_ii],
        [z_ii, z_ii, _sub(Rd, d8, d7), _sub(Rd, d8, d8)],
        [_sub(Rb, b6, b5), _sub(Rb, b6, b6), z_ii, z_ii],
        [z_ii, z_ii, _sub(Rd, d7, d7), _sub(Rd, d7, d8)],
    ])
    D21 = np.block([
        [_sub(Ra, a5, a5), _sub(Ra, a5, a8), z_ii, z_ii],
        [z_ii, z_ii, _sub(Rc, c6, c6), _sub(Rc, c6, c7)],
        [z_ii, z_ii, _sub(Rc, c7, c6), _sub(Rc, c7, c7)],
        [_sub(Ra, a8, a5), _sub(Ra, a8, a8), z_ii, z_ii],
    ])
    h_int = np.concatenate([hb[b5], hd[d8], hb[b6], hd[d7], ha[a5], hc[c6], hc[c7], ha[a8]])
    h_ext = np.concatenate([ha[a1], hb[b2], hc[c3], hd[d4]])
    n = D12.shape[0]
    W = np.eye(n) - D12 @ D21
    Winv = np.linalg.inv(W)
    Dinv = np.zeros((2 * n, 2 * n), dtype=np.complex128)
    Dinv[:n, :n] = Winv
    Dinv[:n, n:] = -Winv @ D12
    Dinv[n:, :n] = -D21 @ Winv
    Dinv[n:, n:] = np.eye(n) + D21 @ Winv @ D12
    S = -Dinv @ C
    T = B @ S
    for k, Ak in enumerate([_sub(Ra, a1, a1), _sub(Rb, b2, b2), _sub(Rc, c3, c3), _sub(Rd, d4, d4)]):
        sl = slice(2 * nc * k, 2 * nc * (k + 1))
        T[sl, sl] += Ak
    g_tilde = -Dinv @ h_int
    h_out = h_ext + B @ g_tilde
    h_out = np.roll(h_out, -nc, axis=0)
    T = np.roll(np.roll(T, -nc, axis=0), -nc, axis=1)
    S = np.roll(S, -nc, axis=1)
    r = np.concatenate([np.arange(0, nc), np.arange(4 * nc, 5 * nc), np.arange(5 * nc, 6 * nc),
                        np.arange(2 * nc, 3 * nc), np.arange(3 * nc, 4 * nc), np.arange(6 * nc, 7 * nc),
                        np.arange(7 * nc, 8 * nc), np.arange(nc, 2 * nc)])
    return S[r], T, h_out, g_tilde[r]


def merge_stage(T, h, L: int, iti: bool = False):
    """Level loop of merge_stage_uniform_2D_{DtN,ItI}
    (merge/_uniform_2D_DtN.py:96-203; merge/_uniform_2D_ItI.py:98-179).

    T: (n_leaves, 4q, 4q); h: (n_leaves, 4q, nsrc).  Returns S_lst,
    g_tilde_lst (leaf-adjacent level first, root last, root with a leading
    batch axis of 1) and the top-level T.
    """
    fn = quad_merge_iti if iti else quad_merge_dtn
    S_lst, g_lst = [], []
    n_levels = max(L, 1)
    for _ in range(n_levels):
        nm = T.shape[0] // 4
        outs = [fn(*T[4 * m:4 * m + 4], *h[4 * m:4 * m + 4]) for m in range(nm)]
        S_lst.append(np.stack([o[0] for o in outs]))
        g_lst.append(np.stack([o[3] for o in outs]))
        T = np.stack([o[1] for o in outs])
        h = np.stack([o[2] for o in outs])
    return S_lst, g_lst, T[0], h[0]


# ---------------------------------------------------------------------------
# Down pass  (src/jaxhps/down_pass/_uniform_2D_DtN.py:7-189,
#             down_pass/_uniform_2D_ItI.py:8-192)
# ---------------------------------------------------------------------------


def _propagate_down_dtn(S, g, gt):
    nc = g.shape[0] // 8
    gi = S @ g + gt
    g5, g6, g7, g8 = gi[:nc], gi[nc:2 * nc], gi[2 * nc:3 * nc], gi[3 * nc:]
    ga = np.concatenate([g[:nc], g5, g8[::-1], g[7 * nc:]])
    gb = np.concatenate([g[nc:3 * nc], g6, g5[::-1]])
    gc = np.concatenate([g6[::-1], g[3 * nc:5 * nc], g7])
    gd = np.concatenate([g8, g7[::-1], g[5 * nc:7 * nc]])
    return np.stack([ga, gb, gc, gd])


def _propagate_down_iti(S, g, gt):
    nc = g.shape[0] // 8
    t = S @ g + gt
    ta5 = t[:nc]
    tb5 = t[nc:2 * nc][::-1]
    tb6 = t[2 * nc:3 * nc]
    tc6 = t[3 * nc:4 * nc][::-1]
    tc7 = t[4 * nc:5 * nc]
    td7 = t[5 * nc:6 * nc][::-1]
    td8 = t[6 * nc:7 * nc]
    ta8 = t[7 * nc:][::-1]
    ga = np.concatenate([g[:nc], ta5, ta8, g[7 * nc:]])
    gb = np.concatenate([g[nc:3 * nc], tb6, tb5])
    gc = np.concatenate([tc6, g[3 * nc:5 * nc], tc7])
    gd = np.concatenate([td8, td7, g[5 * nc:7 * nc]])
    return np.stack([ga, gb, gc, gd])


def down_pass(bdry, S_lst, g_lst, Y, v, iti: bool = False):
    """bdry: (n_bdry, nsrc).  Returns leaf solutions (n_leaves, n_pts, nsrc)."""
    fn = _propagate_down_iti if iti else _propagate_down_dtn
    g = bdry[None]
    for lvl in range(len(S_lst) - 1, -1, -1):
        S, gt = S_lst[lvl], g_lst[lvl]
        g = np.concatenate([fn(S[m], g[m], gt[m]) for m in range(S.shape[0])])
    return np.einsum("ijk,ikl->ijl", Y, g) + v


# ---------------------------------------------------------------------------
# Whole-problem driver (uniform 2D)
# ---------------------------------------------------------------------------


class Problem2D:
    """FP64 oracle problem for a uniform 2D quadtree.

    Coefficient arrays are (n_leaves, p^2) on the leaf points in the
    reference's order; ``source`` is (n_leaves, p^2) or (n_leaves, p^2, nsrc).
    Mirrors PDEProblem (_pdeproblem.py:26-234) for the uniform 2D case.
    """

    OPS = ("D_xx", "D_xy", "D_yy", "D_x", "D_y", "I")

    def __init__(self, root_bounds, L, p, q, coeffs, source, iti=False, eta=None):
        self.root = tuple(float(x) for x in root_bounds)
        self.L, self.p, self.q = L, p, q
        self.iti, self.eta = iti, eta
        self.bounds = uniform_leaf_bounds_2D(self.root, L)
        self.points = leaf_points_2D(self.bounds, p)
        self.boundary_points = boundary_gauss_points_2D(self.root, L, q)
        half = (self.root[1] - self.root[0]) / (2 ** (L + 1))
        dx, dy, dxx, dyy, dxy = diff_operators_2D(p, half)
        self.ops = {"D_xx": dxx, "D_xy": dxy, "D_yy": dyy, "D_x": dx, "D_y": dy,
                    "I": np.eye(p * p)}
        if iti:
            self.P = P_2D_ItI(p, q)
            self.QH = QH_2D_ItI(p, q, dx, dy, eta)
            self.G = G_2D_ItI(dx, dy, p, eta)
        else:
            self.P = P_2D_DtN(p, q)
            self.Q = Q_2D_DtN(p, q, dx, dy)
        self.coeffs = {k: (None if coeffs.get(k) is None else np.asarray(coeffs[k]))
                       for k in self.OPS}
        src = np.asarray(source)
        self.multi = src.ndim == 3
        self.source = src if self.multi else src[..., None]

    def build(self):
        nl = self.bounds.shape[0]
        A = assemble_operator(self.coeffs, self.ops, nl, self.p ** 2)
        if self.iti:
            self.Y, T, self.v, h = leaf_iti(A, self.source, self.P, self.QH, self.G)
        else:
            self.Y, T, self.v, h = leaf_dtn(A, self.source, self.P, self.Q)
        self.T_leaf, self.h_leaf = T, h
        self.S_lst, self.g_lst, self.T_top, self.h_top = merge_stage(T, h, self.L, self.iti)
        return self

    def solve(self, bdry):
        b = np.asarray(bdry)
        b2 = b if b.ndim == 2 else b[:, None]
        u = down_pass(b2, self.S_lst, self.g_lst, self.Y, self.v, self.iti)
        return u if self.multi else u[..., 0]


# ---------------------------------------------------------------------------
# 3D uniform DtN  (src/jaxhps/_grid_creation_3D.py, _precompute_operators_3D.py,
#                  local_solve/_uniform_3D_DtN.py, merge/_uniform_3D_DtN.py,
#                  merge/_schur_complement.py:293-774,
#                  down_pass/_uniform_3D_DtN.py)
# ---------------------------------------------------------------------------


def ext_first_order_3D(p: int) -> np.ndarray:
    """Raster indices (ix p^2 + iy p + iz) in exterior-first order
    (_grid_creation_3D.py:420-458): x faces, then y faces without the x
    faces, then z faces without both, then the interior."""
    idx = np.arange(p ** 3)
    left, right = idx // p ** 2 == 0, idx // p ** 2 == p - 1
    mask = left | right
    bottom = ((idx // p) % p == 0) & ~mask
    top = ((idx // p) % p == p - 1) & ~mask
    mask = mask | bottom | top
    front = (idx % p == 0) & ~mask
    back = (idx % p == p - 1) & ~mask
    mask = mask | front | back
    return np.concatenate([idx[left], idx[right], idx[bottom], idx[top], idx[front], idx[back], idx[~mask]])


def oct_children_bounds(b):
    """Children a..h of an octree node (_grid_creation_3D.py:28-74)."""
    x0, x1, y0, y1, z0, z1 = b
    xm, ym, zm = (x0 + x1) / 2, (y0 + y1) / 2, (z0 + z1) / 2
    return np.array([
        [x0, xm, y0, ym, zm, z1], [xm, x1, y0, ym, zm, z1], [xm, x1, ym, y1, zm, z1], [x0, xm, ym, y1, zm, z1],
        [x0, xm, y0, ym, z0, zm], [xm, x1, y0, ym, z0, zm], [xm, x1, ym, y1, z0, zm], [x0, xm, ym, y1, z0, zm],
    ])


def uniform_leaf_bounds_3D(root_bounds, L: int) -> np.ndarray:
    b = np.asarray([root_bounds], dtype=np.float64)
    for _ in range(L):
        b = np.concatenate([oct_children_bounds(x) for x in b])
    return b


def leaf_points_3D(bounds: np.ndarray, p: int) -> np.ndarray:
    """meshgrid(x, y, z, 'ij') then exterior-first (_grid_creation_3D.py:77-116)."""
    c = chebyshev_points(p)
    r = ext_first_order_3D(p)
    out = []
    for b in np.atleast_2d(bounds):
        X, Y, Z = np.meshgrid(affine_transform(c, b[0:2]), affine_transform(c, b[2:4]),
                              affine_transform(c, b[4:6]), indexing="ij")
        out.append(np.stack([X.ravel(), Y.ravel(), Z.ravel()], -1)[r])
    return np.stack(out)


def boundary_gauss_points_3D(root_bounds, L: int, q: int) -> np.ndarray:
    """Root boundary Gauss points (_grid_creation_3D.py:119-236): each face's
    panel list is the 2D quad subdivision of its two coordinates repeated L
    times; Gauss points meshgrid 'ij' inside a panel."""
    x0, x1, y0, y1, z0, z1 = root_bounds
    g = gauss_points(q)

    def panels(u0, u1, v0, v1):
        b = np.array([[u0, u1, v0, v1]])
        for _ in range(L):
            b = np.concatenate([quad_children_bounds(x) for x in b])
        pts = []
        for u0_, u1_, v0_, v1_ in b:
            U, V = np.meshgrid(affine_transform(g, (u0_, u1_)), affine_transform(g, (v0_, v1_)), indexing="ij")
            pts.append(np.stack([U.ravel(), V.ravel()], -1))
        return np.concatenate(pts)

    yz, xz, xy = panels(y0, y1, z0, z1), panels(x0, x1, z0, z1), panels(x0, x1, y0, y1)
    n = yz.shape[0]
    f = [np.column_stack([np.full(n, x0), yz]), np.column_stack([np.full(n, x1), yz]),
         np.column_stack([xz[:, 0], np.full(n, y0), xz[:, 1]]), np.column_stack([xz[:, 0], np.full(n, y1), xz[:, 1]]),
         np.column_stack([xy, np.full(n, z0)]), np.column_stack([xy, np.full(n, z1)])]
    return np.concatenate(f)


def face_idxes_3D(p: int, face: int) -> np.ndarray:
    """get_face_1_idxes .. get_face_6_idxes (_precompute_operators_3D.py:220-320),
    ``face`` = 0..5 for the reference's faces 1..6."""
    if face == 0:
        return np.arange(p ** 2)
    if face == 1:
        return np.arange(p ** 2) + p ** 2
    if face == 2:
        return np.concatenate([np.arange(p), np.arange(2 * p ** 2, 3 * p ** 2 - 2 * p), np.arange(p ** 2, p ** 2 + p)])
    if face == 3:
        return np.concatenate([np.arange(p * (p - 1), p ** 2), np.arange(3 * p ** 2 - 2 * p, 4 * p ** 2 - 4 * p),
                               np.arange(2 * p ** 2 - p, 2 * p ** 2)])
    if face == 4:
        first_col = np.arange(0, p ** 2, p)
        last_col = np.arange(p ** 2, 2 * p ** 2, p)
        first_row = np.arange(2 * p ** 2, 3 * p ** 2 - 2 * p, p)
        last_row = np.arange(3 * p ** 2 - 2 * p, 4 * p ** 2 - 4 * p, p)
        interior = np.arange(4 * p ** 2 - 4 * p, 4 * p ** 2 - 4 * p + (p - 2) ** 2)
    else:
        first_col = np.arange(p - 1, p ** 2, p)
        last_col = np.arange(p ** 2 + p - 1, 2 * p ** 2, p)
        first_row = np.arange(2 * p ** 2 + p - 1, 3 * p ** 2 - 2 * p, p)
        last_row = np.arange(3 * p ** 2 - 2 * p + p - 1, 4 * p ** 2 - 4 * p, p)
        u = p ** 3 - (p - 2) ** 3
        interior = np.arange(u - (p - 2) ** 2, u)
    out = [first_col]
    for i in range(p - 2):
        out += [first_row[i:i + 1], interior[i * (p - 2):(i + 1) * (p - 2)], last_row[i:i + 1]]
    out.append(last_col)
    return np.concatenate(out)


def diff_operators_3D(p: int, half_side_len: float):
    """(_precompute_operators_3D.py:17-61) -> dx, dy, dz, dxx, dyy, dzz, dxy, dxz, dyz."""
    r = ext_first_order_3D(p)
    D = differentiation_matrix_1D(chebyshev_points(p)) / half_side_len
    I = np.eye(p)
    dx = np.kron(D, np.kron(I, I))[r][:, r]
    dy = np.kron(I, np.kron(D, I))[r][:, r]
    dz = np.kron(I, np.kron(I, D))[r][:, r]
    return dx, dy, dz, dx @ dx, dy @ dy, dz @ dz, dx @ dy, dx @ dz, dy @ dz


def _bary2D(fx, fy, tx, ty):
    return np.kron(barycentric_matrix_1D(fx, tx), barycentric_matrix_1D(fy, ty))


def P_3D_DtN(p: int, q: int) -> np.ndarray:
    """(_precompute_operators_3D.py:64-147): per-face 2D interpolation, the 8
    corner rows divided by 3 and the 12 edge row ranges divided by 2."""
    g, c = gauss_points(q), chebyshev_points(p)
    B = _bary2D(g, g, c, c)
    P = np.zeros((p ** 3 - (p - 2) ** 3, 6 * q ** 2))
    for f in range(6):
        P[face_idxes_3D(p, f), f * q ** 2:(f + 1) * q ** 2] = B
    corners = np.array([0, p - 1, p ** 2 - p, p ** 2 - 1, p ** 2, p ** 2 + p - 1, 2 * p ** 2 - p, 2 * p ** 2 - 1])
    P[corners] /= 3
    edges = np.concatenate([
        np.arange(1, p - 1), np.arange(p ** 2 + 1, p ** 2 + p - 1), np.arange(p ** 2 - p + 1, p ** 2 - 1),
        np.arange(2 * p ** 2 - p + 1, 2 * p ** 2 - 1), np.arange(1, p - 1) * p, np.arange(p, p ** 2 - p, p) + p ** 2,
        np.arange(2 * p ** 2, 3 * p ** 2 - 2 * p, p), np.arange(3 * p ** 2 - 2 * p, 4 * p ** 2 - 4 * p, p),
        np.arange(2 * p - 1, p ** 2 - p, p), np.arange(p ** 2 + 2 * p - 1, 2 * p ** 2 - p, p),
        np.arange(2 * p ** 2 + p - 1, 3 * p ** 2 - 2 * p, p), np.arange(3 * p ** 2 - 2 * p + p - 1, 4 * p ** 2 - 4 * p, p),
    ])
    P[edges] /= 2
    return P


def Q_3D_DtN(p: int, q: int, dx, dy, dz) -> np.ndarray:
    """(_precompute_operators_3D.py:150-210): N rows = -/+ d/dn on each face,
    then kron(I_6, cheby->gauss 2D interpolation) @ N."""
    N = np.concatenate([-dx[face_idxes_3D(p, 0)], dx[face_idxes_3D(p, 1)], -dy[face_idxes_3D(p, 2)],
                        dy[face_idxes_3D(p, 3)], -dz[face_idxes_3D(p, 4)], dz[face_idxes_3D(p, 5)]])
    g, c = gauss_points(q), chebyshev_points(p)
    return np.kron(np.eye(6), _bary2D(c, c, g, g)) @ N


# Oct merge bookkeeping (merge/_uniform_3D_DtN.py:190-380): for each child
# a..h, the faces (0..5 = reference faces 1..6) forming its part of the merged
# exterior, and its three interfaces as (label, face).  Labels 9..20 are the
# reference's interface numbers.
_OCT_CHILD = (
    ((0, 2, 5), ((9, 1), (12, 3), (17, 4))),     # a
    ((1, 2, 5), ((9, 0), (10, 3), (18, 4))),     # b
    ((1, 3, 5), ((10, 2), (11, 0), (19, 4))),    # c
    ((0, 3, 5), ((11, 1), (12, 2), (20, 4))),    # d
    ((0, 2, 4), ((13, 1), (16, 3), (17, 5))),    # e
    ((1, 2, 4), ((13, 0), (14, 3), (18, 5))),    # f
    ((1, 3, 4), ((14, 2), (15, 0), (19, 5))),    # g
    ((0, 3, 4), ((15, 1), (16, 2), (20, 5))),    # h
)
# Merged-face assembly order of the children's sub-blocks (get_rearrange_indices, :442-541).
_OCT_FACE_CHILDREN = ((4, 7, 3, 0), (5, 6, 2, 1), (4, 5, 1, 0), (7, 6, 2, 3), (4, 5, 6, 7), (0, 1, 2, 3))


def oct_merge_dtn(Ts, hs):
    """One DtN oct merge (merge/_uniform_3D_DtN.py:127-187 with
    _schur_complement.py:293-774 and the re-ordering of :442-541).

    Ts: 8 child T (6nf, 6nf); hs: 8 child h (6nf, nsrc).  Returns S, T,
    h_out, g_tilde, all in the reference's final orders."""
    nf = Ts[0].shape[0] // 6
    ix = np.arange(6 * nf)

    def face(f):
        return ix[f * nf:(f + 1) * nf]

    ext_sets = [np.concatenate([face(f) for f in ch[0]]) for ch in _OCT_CHILD]
    int_sets = [{lab: face(f) for lab, f in ch[1]} for ch in _OCT_CHILD]
    n_ext, n_int = 24 * nf, 12 * nf
    dt = np.result_type(*Ts)
    B = np.zeros((n_ext, n_int), dtype=dt)
    C = np.zeros((n_int, n_ext), dtype=dt)
    D = np.zeros((n_int, n_int), dtype=dt)
    ns = hs[0].shape[1]
    dh = np.zeros((n_int, ns), dtype=dt)
    h_ext = np.zeros((n_ext, ns), dtype=dt)

    def isl(lab):
        return slice((lab - 9) * nf, (lab - 8) * nf)

    for c in range(8):
        es = slice(3 * nf * c, 3 * nf * (c + 1))
        h_ext[es] = hs[c][ext_sets[c]]
        for lab, idx in int_sets[c].items():
            B[es, isl(lab)] = Ts[c][np.ix_(ext_sets[c], idx)]
            C[isl(lab), es] = Ts[c][np.ix_(idx, ext_sets[c])]
            dh[isl(lab)] += hs[c][idx]
            for lab2, idx2 in int_sets[c].items():
                D[isl(lab), isl(lab2)] += Ts[c][np.ix_(idx, idx2)]
    Dinv = np.linalg.inv(D)
    S = -Dinv @ C
    T = B @ S
    for c in range(8):
        es = slice(3 * nf * c, 3 * nf * (c + 1))
        T[es, es] += Ts[c][np.ix_(ext_sets[c], ext_sets[c])]
    g_tilde = -Dinv @ dh
    h_out = h_ext + B @ g_tilde
    # region c = [x-face block, y-face block, z-face block] of 3 nf each
    r = []
    for F, kids in enumerate(_OCT_FACE_CHILDREN):
        for c in kids:
            r.append(np.arange(3 * nf * c + (F // 2) * nf, 3 * nf * c + (F // 2 + 1) * nf))
    r = np.concatenate(r)
    return S[:, r], T[np.ix_(r, r)], h_out[r], g_tilde


def merge_stage_3D(T, h, L: int):
    """Level loop of merge_stage_uniform_3D_DtN (merge/_uniform_3D_DtN.py:12-124)."""
    S_lst, g_lst = [], []
    for _ in range(L):
        nm = T.shape[0] // 8
        outs = [oct_merge_dtn(T[8 * m:8 * m + 8], h[8 * m:8 * m + 8]) for m in range(nm)]
        S_lst.append(np.stack([o[0] for o in outs]))
        g_lst.append(np.stack([o[3] for o in outs]))
        T = np.stack([o[1] for o in outs])
        h = np.stack([o[2] for o in outs])
    # the root entries are stored without a batch axis (merge/_uniform_3D_DtN.py:116)
    S_lst[-1], g_lst[-1] = S_lst[-1][0], g_lst[-1][0]
    return S_lst, g_lst, T[0], h[0]


# Child boundary assembly of _propogate_down_oct_DtN (down_pass/_uniform_3D_DtN.py:116-246):
# per child, per own face, either ("b", merged face, block) or ("i", label).
_OCT_DOWN = (
    (("b", 0, 3), ("i", 9), ("b", 2, 3), ("i", 12), ("i", 17), ("b", 5, 0)),
    (("i", 9), ("b", 1, 3), ("b", 2, 2), ("i", 10), ("i", 18), ("b", 5, 1)),
    (("i", 11), ("b", 1, 2), ("i", 10), ("b", 3, 2), ("i", 19), ("b", 5, 2)),
    (("b", 0, 2), ("i", 11), ("i", 12), ("b", 3, 3), ("i", 20), ("b", 5, 3)),
    (("b", 0, 0), ("i", 13), ("b", 2, 0), ("i", 16), ("b", 4, 0), ("i", 17)),
    (("i", 13), ("b", 1, 0), ("b", 2, 1), ("i", 14), ("b", 4, 1), ("i", 18)),
    (("i", 15), ("b", 1, 1), ("i", 14), ("b", 3, 1), ("b", 4, 2), ("i", 19)),
    (("b", 0, 1), ("i", 15), ("i", 16), ("b", 3, 0), ("b", 4, 3), ("i", 20)),
)


def _propagate_down_oct(S, g, gt):
    nf = g.shape[0] // 24
    gi = S @ g + gt
    out = []
    for spec in _OCT_DOWN:
        parts = []
        for s in spec:
            if s[0] == "b":
                o = s[1] * 4 * nf + s[2] * nf
                parts.append(g[o:o + nf])
            else:
                parts.append(gi[(s[1] - 9) * nf:(s[1] - 8) * nf])
        out.append(np.concatenate(parts))
    return np.stack(out)


def down_pass_3D(bdry, S_lst, g_lst, Y, v):
    """down_pass/_uniform_3D_DtN.py:8-113; the root entries are expanded (:86-87)."""
    S_lst = list(S_lst[:-1]) + [S_lst[-1][None]]
    g_lst = list(g_lst[:-1]) + [g_lst[-1][None]]
    g = bdry[None]
    for lvl in range(len(S_lst) - 1, -1, -1):
        S, gt = S_lst[lvl], g_lst[lvl]
        g = np.concatenate([_propagate_down_oct(S[m], g[m], gt[m]) for m in range(S.shape[0])])
    return np.einsum("ijk,ikl->ijl", Y, g) + v


class Problem3D:
    """FP64 oracle problem for a uniform 3D octree (DtN).  Coefficients are
    (n_leaves, p^3) arrays on the leaf points; ``source`` (n_leaves, p^3[, nsrc])."""

    OPS = ("D_xx", "D_xy", "D_yy", "D_xz", "D_yz", "D_zz", "D_x", "D_y", "D_z", "I")

    def __init__(self, root_bounds, L, p, q, coeffs, source):
        self.root = tuple(float(x) for x in root_bounds)
        self.L, self.p, self.q = L, p, q
        self.bounds = uniform_leaf_bounds_3D(self.root, L)
        self.points = leaf_points_3D(self.bounds, p)
        self.boundary_points = boundary_gauss_points_3D(self.root, L, q)
        half = (self.root[1] - self.root[0]) / (2 ** (L + 1))
        dx, dy, dz, dxx, dyy, dzz, dxy, dxz, dyz = diff_operators_3D(p, half)
        self.ops = {"D_xx": dxx, "D_xy": dxy, "D_yy": dyy, "D_xz": dxz, "D_yz": dyz, "D_zz": dzz,
                    "D_x": dx, "D_y": dy, "D_z": dz, "I": np.eye(p ** 3)}
        self.P = P_3D_DtN(p, q)
        self.Q = Q_3D_DtN(p, q, dx, dy, dz)
        self.coeffs = {k: (None if coeffs.get(k) is None else np.asarray(coeffs[k])) for k in self.OPS}
        src = np.asarray(source)
        self.multi = src.ndim == 3
        self.source = src if self.multi else src[..., None]

    def build(self):
        nl = self.bounds.shape[0]
        A = assemble_operator(self.coeffs, self.ops, nl, self.p ** 3)
        self.Y, T, self.v, h = leaf_dtn(A, self.source, self.P, self.Q)
        self.T_leaf, self.h_leaf = T, h
        self.S_lst, self.g_lst, self.T_top, self.h_top = merge_stage_3D(T, h, self.L)
        return self

    def solve(self, bdry):
        b = np.asarray(bdry)
        b2 = b if b.ndim == 2 else b[:, None]
        u = down_pass_3D(b2, self.S_lst, self.g_lst, self.Y, self.v)
        return u if self.multi else u[..., 0]


# ---------------------------------------------------------------------------
# Adaptive octree meshing  (src/jaxhps/_adaptive_discretization_3D.py:34-503,
#                           _discretization_tree_operations_3D.py:26-98,
#                           _precompute_operators_3D.py:412-500)
# ---------------------------------------------------------------------------


def chebyshev_weights(n: int, bounds) -> np.ndarray:
    """Clenshaw-Curtis weights on [a, b] (quadrature/_discretization.py:40-86)."""
    a, b = bounds
    c = 2.0 / np.concatenate([[1.0], 1.0 - np.arange(2, n, 2) ** 2])
    start = n // 2 if n % 2 else n // 2 + 1
    c = np.concatenate([c, np.flip(c[1:start])])
    w = np.fft.ifft(c).real
    out = np.concatenate([w, [w[0] / 2]])
    out[0] = w[0] / 2
    return out * (b - a) / 2


def L_8f1(p: int) -> np.ndarray:
    """Dense node -> eight children interpolation, rows blocks a..h each in
    exterior-first order, columns exterior-first (_precompute_operators_3D.py
    :412-500)."""
    c = chebyshev_points(p)
    lo, hi = affine_transform(c, (-1.0, 0.0)), affine_transform(c, (0.0, 1.0))
    Bl, Bh = barycentric_matrix_1D(c, lo), barycentric_matrix_1D(c, hi)
    r = ext_first_order_3D(p)
    bits = ((0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1), (0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0))
    blocks = []
    for bx, by, bz in bits:
        M = np.kron(np.kron(Bh if bx else Bl, Bh if by else Bl), Bh if bz else Bl)
        blocks.append(M[r][:, r])
    return np.concatenate(blocks)


class OctNode:
    """Minimal octree node for the oracle (bounds, depth, children, face counts)."""

    def __init__(self, bounds, depth=0):
        self.b = tuple(float(x) for x in bounds)
        self.depth = depth
        self.children = []
        self.n = [None] * 6

    def leaves(self):
        if not self.children:
            return [self]
        out = []
        for ch in self.children:
            out += ch.leaves()
        return out


def oracle_add_eight_children(node: OctNode, root: OctNode = None, q: int = None):
    """_discretization_tree_operations_3D.py:26-98."""
    if node.children:
        return
    node.children = [OctNode(b, node.depth + 1) for b in oct_children_bounds(node.b)]
    if q is None:
        return
    q2 = q * q
    for ch in node.children:
        ch.n = [q2] * 6
    node.n = [4 * q2] * 6
    if root is None or node is root:
        return
    cur = root
    while node not in cur.children:   # ancestors from the root to the parent
        for k in range(6):
            if cur.b[k] == node.b[k]:
                cur.n[k] += 3 * q2
        xm, ym, zm = (cur.b[0] + cur.b[1]) / 2, (cur.b[2] + cur.b[3]) / 2, (cur.b[4] + cur.b[5]) / 2
        x0, y0, z0 = node.b[0], node.b[2], node.b[4]
        if x0 < xm:
            i = (4 if z0 < zm else 0) if y0 < ym else (7 if z0 < zm else 3)
        else:
            i = (5 if z0 < zm else 1) if y0 < ym else (6 if z0 < zm else 2)
        cur = cur.children[i]
    for k in range(6):
        if cur.b[k] == node.b[k]:
            cur.n[k] += 3 * q2


def _oracle_volumes(n: OctNode, root: OctNode):
    s = n.b[1] - n.b[0]
    x0, x1, y0, y1, z0, z1 = n.b
    v = []
    if x0 - s >= root.b[0]:
        v.append((x0 - s, x0, y0, y1, z0, z1))
    if x1 + s <= root.b[1]:
        v.append((x1, x1 + s, y0, y1, z0, z1))
    if y0 - s >= root.b[2]:
        v.append((x0, x1, y0 - s, y0, z0, z1))
    if y1 + s <= root.b[3]:
        v.append((x0, x1, y1, y1 + s, z0, z1))
    if z0 - s >= root.b[4]:
        v.append((x0, x1, y0, y1, z0 - s, z0))
    if z1 + s <= root.b[5]:
        v.append((x0, x1, y0, y1, z1, z1 + s))
    return v


def _oracle_find_or_add(node: OctNode, root: OctNode, q, vol):
    """find_or_add_child (_adaptive_discretization_3D.py:317-420)."""
    xmin, xmax, ymin, ymax, zmin, zmax = vol
    side = node.b[1] - node.b[0]
    req = xmax - xmin
    if np.allclose(req * 2, side):
        if not node.children:
            oracle_add_eight_children(node, root, q)
            return node
        return None
    xm, ym, zm = (node.b[0] + node.b[1]) / 2, (node.b[2] + node.b[3]) / 2, (node.b[4] + node.b[5]) / 2
    if xmin < xm:
        i = (4 if zmin < zm else 0) if ymin < ym else (7 if zmin < zm else 3)
    else:
        i = (5 if zmin < zm else 1) if ymin < ym else (6 if zmin < zm else 2)
    child = node.children[i]
    if np.allclose(side, 4 * req):
        if not child.children:
            oracle_add_eight_children(child, root, q)
            return child
        return None
    if side < 2 * req:
        raise ValueError("Requested volume is too large for the current node")
    return _oracle_find_or_add(child, root, q, vol)


def oracle_adaptive_mesh_3D(root: OctNode, f, tol: float, p: int, q: int, restrict: bool = True,
                            l2: bool = False):
    """generate_adaptive_mesh_level_restriction (_adaptive_discretization_3D.py:34-210)
    with the dense L_8f1 check; ``f`` takes (..., 3) NumPy points.  Refines in
    place; returns the number of rounds."""
    Lop = L_8f1(p)
    r = ext_first_order_3D(p)

    def sq_l2(vals, b):
        w = np.einsum("i,j,k->ijk", chebyshev_weights(p, b[0:2]), chebyshev_weights(p, b[2:4]),
                      chebyshev_weights(p, b[4:6])).ravel()[r]
        return float(np.sum(w * vals ** 2))

    if l2:
        oracle_add_eight_children(root, root, q)
        gn = sum(sq_l2(f(leaf_points_3D(np.array([lf.b]), p)[0]), lf.b) for lf in root.leaves())
        tol = tol ** 2
    else:
        gn = float(np.max(f(leaf_points_3D(oct_children_bounds(root.b), p).reshape(-1, 3))))
    queue = root.leaves()
    rounds = 0
    while queue:
        rounds += 1
        ok, nrms = [], []
        for node in queue:
            f0 = f(leaf_points_3D(np.array([node.b]), p)[0])
            f1 = f(leaf_points_3D(oct_children_bounds(node.b), p).reshape(-1, 3))
            d = Lop @ f0 - f1
            if l2:
                kids = oct_children_bounds(node.b)
                err = sum(sq_l2(d[k * p ** 3:(k + 1) * p ** 3], kids[k]) for k in range(8))
                ok.append(err / gn < tol)
                nrms.append(0.0)
            else:
                nrm = max(gn, float(np.max(np.abs(f1))))
                ok.append(float(np.max(np.abs(d))) / nrm < tol)
                nrms.append(nrm)
        if not l2:
            gn = max(nrms)
        new_queue = []
        for node, good in zip(queue, ok):
            if good:
                continue
            oracle_add_eight_children(node, root, q)
            new_queue += node.children
            if restrict:
                pending = [node]
                while pending:
                    fc = pending.pop()
                    for vol in _oracle_volumes(fc, root):
                        n = _oracle_find_or_add(root, root, q, vol)
                        if n is not None:
                            pending.append(n)
                            new_queue += n.children
        queue = new_queue
    return rounds


# ---------------------------------------------------------------------------
# Refinement-proposal MLP (no reference counterpart): 513 -> 64 -> 64 -> 1,
# ReLU, weighted binary cross-entropy with logits, Adam.
# ---------------------------------------------------------------------------


def mlp_unpack(params: np.ndarray):
    p = np.asarray(params, dtype=np.float64)
    o = 0
    out = []
    for shape in ((64, 513), (64,), (64, 64), (64,), (64,), (1,)):
        n = int(np.prod(shape))
        out.append(p[o:o + n].reshape(shape))
        o += n
    return out


def mlp_forward(params, X):
    W1, b1, W2, b2, w3, b3 = mlp_unpack(params)
    H1 = np.maximum(X @ W1.T + b1, 0.0)
    H2 = np.maximum(H1 @ W2.T + b2, 0.0)
    return H2 @ w3 + b3[0], H1, H2


def mlp_loss(params, X, y, pos_weight=1.0):
    z, _, _ = mlp_forward(params, X)
    w = np.where(y > 0.5, pos_weight, 1.0)
    return float(np.mean(w * (np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))))


def mlp_grad(params, X, y, pos_weight=1.0):
    """Gradient of mlp_loss by back-propagation, packed like the parameters."""
    W1, b1, W2, b2, w3, b3 = mlp_unpack(params)
    z, H1, H2 = mlp_forward(params, X)
    n = X.shape[0]
    w = np.where(y > 0.5, pos_weight, 1.0)
    dz = w * (1.0 / (1.0 + np.exp(-z)) - y) / n
    gw3 = H2.T @ dz
    gb3 = np.array([dz.sum()])
    d2 = np.outer(dz, w3) * (H2 > 0)
    gW2 = d2.T @ H1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (H1 > 0)
    gW1 = d1.T @ X
    gb1 = d1.sum(0)
    return np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, gb3])


def adam_step(params, grad, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad ** 2
    p = params - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v


# ---------------------------------------------------------------------------
# Adaptive 3D DtN build/solve  (local_solve/_adaptive_3D_DtN.py:13-175,
#   merge/_adaptive_3D_DtN.py:30-565, merge/_utils_adaptive_3D_DtN.py:11-881,
#   down_pass/_adaptive_3D_DtN.py:15-394) on OctNode trees whose face counts
#   ``n`` were kept by oracle_add_eight_children.
# ---------------------------------------------------------------------------

_FACE_ORDERS = ((4, 7, 3, 0, 5, 6, 2, 1), (4, 5, 1, 0, 7, 6, 2, 3), (0, 1, 2, 3, 4, 5, 6, 7))


def oracle_face_leaves(node: OctNode):
    """get_ordered_lst_of_boundary_nodes (_grid_creation_3D.py:375-417)."""
    def walk(n, order):
        if not n.children:
            return [n]
        out = []
        for i in order:
            out += walk(n.children[i], order)
        return out
    return [[lf for lf in walk(node, _FACE_ORDERS[f // 2]) if lf.b[f] == node.b[f]] for f in range(6)]


def oracle_projection_lst(l0, l1):
    """merge/_utils_adaptive_3D_DtN.py:11-57."""
    o0, o1 = [], []
    i0 = i1 = 0
    while i0 < len(l0) and i1 < len(l1):
        s0, s1 = l0[i0].b[1] - l0[i0].b[0], l1[i1].b[1] - l1[i1].b[0]
        if s0 == s1:
            o0.append(False), o1.append(False)
            i0 += 1
            i1 += 1
        elif s0 < s1:
            o0 += [True] * 4
            o1.append(False)
            i0 += 4
            i1 += 1
        else:
            o1 += [True] * 4
            o0.append(False)
            i1 += 4
            i0 += 1
    return o0, o1


def _compress_rows(T, L, flags):
    """_compress_rows_from_lst (:676-711): groups of 4 panels -> L @ rows."""
    npp = L.shape[0]
    out, i = [], 0
    while i < len(flags):
        if flags[i]:
            out.append(L @ T[i * npp:(i + 4) * npp])
            i += 4
        else:
            out.append(T[i * npp:(i + 1) * npp])
            i += 1
    return np.concatenate(out, axis=0)


def _compress_cols(T, L, flags):
    """_compress_cols_from_lst (:647-674): groups of 4 panels -> cols @ L."""
    npp = L.shape[1]
    out, i = [], 0
    while i < len(flags):
        if flags[i]:
            out.append(T[:, i * npp:(i + 4) * npp] @ L)
            i += 4
        else:
            out.append(T[:, i * npp:(i + 1) * npp])
            i += 1
    return np.concatenate(out, axis=1)


def _deproject(g, L, flags, npp):
    """Inverse direction of one interface side (_deproject_merge_interface_3D)."""
    out, i, k = [], 0, 0
    while i < len(flags):
        seg = g[k:k + npp]
        if flags[i]:
            out.append(L @ seg)
            i += 4
        else:
            out.append(seg)
            i += 1
        k += npp
    return np.concatenate(out, axis=0), k


def _label_pairs():
    """label -> ((child, face), (child, face)) from the _OCT_CHILD table."""
    pairs = {}
    for c, (_, ints) in enumerate(_OCT_CHILD):
        for lab, f in ints:
            pairs.setdefault(lab, []).append((c, f))
    return pairs


def oracle_adaptive_oct_merge(node: OctNode, L_4f1, L_1f4):
    kids = node.children
    fl = [oracle_face_leaves(k) for k in kids]
    pairs = _label_pairs()
    flags = {}
    for lab in range(9, 21):
        (c0, f0), (c1, f1) = pairs[lab]
        a, b = oracle_projection_lst(fl[c0][f0], fl[c1][f1])
        flags[(c0, lab)], flags[(c1, lab)] = a, b
    ns = kids[0].h.shape[1]
    subs = []
    for c, (ext_faces, ints) in enumerate(_OCT_CHILD):
        n = kids[c].n
        off = np.concatenate([[0], np.cumsum(n)])
        sets = [np.concatenate([np.arange(off[f], off[f + 1]) for f in ext_faces])] + \
               [np.arange(off[f], off[f + 1]) for _, f in ints]
        labs = [None] + [lab for lab, _ in ints]
        blk = {}
        for i, (ri, rl) in enumerate(zip(sets, labs)):
            for j, (ci, cl) in enumerate(zip(sets, labs)):
                M = kids[c].T[np.ix_(ri, ci)]
                if rl is not None and any(flags[(c, rl)]):
                    M = _compress_rows(M, L_1f4, flags[(c, rl)])
                if cl is not None and any(flags[(c, cl)]):
                    M = _compress_cols(M, L_4f1, flags[(c, cl)])
                blk[(rl, cl)] = M
            v = kids[c].h[ri]
            if rl is not None and any(flags[(c, rl)]):
                v = _compress_rows(v, L_1f4, flags[(c, rl)])
            blk[("h", rl)] = v
        subs.append(blk)
    msz = {lab: subs[pairs[lab][0][0]][(lab, lab)].shape[0] for lab in range(9, 21)}
    ioff = dict(zip(range(9, 21), np.concatenate([[0], np.cumsum([msz[l] for l in range(9, 21)])])))
    esz = [subs[c][(None, None)].shape[0] for c in range(8)]
    eoff = np.concatenate([[0], np.cumsum(esz)])
    n_ext, n_int = int(eoff[-1]), int(sum(msz.values()))
    B = np.zeros((n_ext, n_int))
    Cm = np.zeros((n_int, n_ext))
    D = np.zeros((n_int, n_int))
    dh = np.zeros((n_int, ns))
    hx = np.zeros((n_ext, ns))
    A = np.zeros((n_ext, n_ext))
    for c, (_, ints) in enumerate(_OCT_CHILD):
        es = slice(eoff[c], eoff[c + 1])
        A[es, es] = subs[c][(None, None)]
        hx[es] = subs[c][("h", None)]
        for lab, _ in ints:
            ls = slice(ioff[lab], ioff[lab] + msz[lab])
            B[es, ls] = subs[c][(None, lab)]
            Cm[ls, es] = subs[c][(lab, None)]
            dh[ls] += subs[c][("h", lab)]
            for lab2, _ in ints:
                D[ls, slice(ioff[lab2], ioff[lab2] + msz[lab2])] += subs[c][(lab, lab2)]
    Dinv = np.linalg.inv(D)
    S = -Dinv @ Cm
    T = A + B @ S
    gt = -Dinv @ dh
    h_out = hx + B @ gt
    # re-order the regions [x-face, y-face, z-face] of a..h into faces 0..5 (:745-881)
    r = []
    for F, order in enumerate(_OCT_FACE_CHILDREN):
        for c in order:
            faces = _OCT_CHILD[c][0]
            k = faces.index(F)
            start = eoff[c] + sum(kids[c].n[f] for f in faces[:k])
            r.append(np.arange(start, start + kids[c].n[F]))
    r = np.concatenate(r)
    return S[:, r], T[np.ix_(r, r)], h_out[r], gt, flags, msz


def oracle_adaptive_build_3D(root: OctNode, p: int, q: int, coeffs: dict, source):
    """Leaf stage with per-leaf rescaled operators and Q / h, then merges
    from the deepest level up (merge_stage_adaptive_3D_DtN, :30-149)."""
    leaves = root.leaves()
    dx, dy, dz, dxx, dyy, dzz, dxy, dxz, dyz = diff_operators_3D(p, 1.0)
    ops = {"D_xx": dxx, "D_xy": dxy, "D_yy": dyy, "D_xz": dxz, "D_yz": dyz, "D_zz": dzz, "D_x": dx, "D_y": dy,
           "D_z": dz, "I": np.eye(p ** 3)}
    order = {"D_xx": 2, "D_xy": 2, "D_yy": 2, "D_xz": 2, "D_yz": 2, "D_zz": 2, "D_x": 1, "D_y": 1, "D_z": 1, "I": 0}
    P = P_3D_DtN(p, q)
    Q = Q_3D_DtN(p, q, dx, dy, dz)
    src = np.asarray(source)
    src = src if src.ndim == 3 else src[..., None]
    for i, lf in enumerate(leaves):
        h = (lf.b[1] - lf.b[0]) / 2
        A = sum(np.asarray(coeffs[k])[i][:, None] * ops[k] / h ** order[k] for k in coeffs if coeffs[k] is not None)
        Y, T, v, hv = leaf_dtn(A[None], src[i:i + 1], P, Q / h)
        lf.Y, lf.T, lf.v, lf.h = Y[0], T[0], v[0], hv[0]
    g = q * q
    gq = gauss_points(q)
    lo, hi = affine_transform(gq, (-1.0, 0.0)), affine_transform(gq, (0.0, 1.0))
    quarters = ((lo, lo), (hi, lo), (hi, hi), (lo, hi))
    L_4f1 = np.concatenate([_bary2D(gq, gq, u, v) for u, v in quarters])
    L_1f4 = np.zeros((g, 4 * g))
    for k, (u, v) in enumerate(quarters):
        rows = (((gq < 0) if u is lo else (gq >= 0))[:, None] & ((gq < 0) if v is lo else (gq >= 0))[None, :]).ravel()
        L_1f4[rows, k * g:(k + 1) * g] = _bary2D(u, v, gq, gq)[rows]

    def merge(node):
        for ch in node.children:
            if ch.children:
                merge(ch)
        node.S, node.T, node.h, node.gt, node.flags, node.msz = oracle_adaptive_oct_merge(node, L_4f1, L_1f4)

    merge(root)
    root.L_4f1 = L_4f1
    return root


def oracle_adaptive_solve_3D(root: OctNode, bdry):
    """down_pass_adaptive_3D_DtN (:15-142, _propagate_down_oct :176-394)."""
    L_4f1 = root.L_4f1
    g_all = np.asarray(bdry)
    root.g = g_all if g_all.ndim == 2 else g_all[:, None]
    pairs = _label_pairs()

    def down(node):
        if not node.children:
            return
        kids = node.children
        gi = node.S @ node.g + node.gt
        foff = np.concatenate([[0], np.cumsum(node.n)])
        faces = [node.g[foff[f]:foff[f + 1]] for f in range(6)]
        ioff = np.concatenate([[0], np.cumsum([node.msz[l] for l in range(9, 21)])])
        iface = {}
        npp = L_4f1.shape[1]
        for k, lab in enumerate(range(9, 21)):
            seg = gi[ioff[k]:ioff[k + 1]]
            for c, f in pairs[lab]:
                iface[(c, f)] = _deproject(seg, L_4f1, node.flags[(c, lab)], npp)[0]
        for c, ch in enumerate(kids):
            parts = []
            for f in range(6):
                if (c, f) in iface:
                    parts.append(iface[(c, f)])
                else:
                    order = _OCT_FACE_CHILDREN[f]
                    start = sum(kids[o].n[f] for o in order[:order.index(c)])
                    parts.append(faces[f][start:start + ch.n[f]])
            ch.g = np.concatenate(parts)
            down(ch)

    down(root)
    return np.stack([lf.Y @ lf.g + lf.v for lf in root.leaves()])


# ---------------------------------------------------------------------------
# Interpolation between the HPS grid and rectangular grids
# (src/jaxhps/_interpolation_methods.py:23-340,
#  quadrature/_interpolation.py:117-320)
# ---------------------------------------------------------------------------

_EPS = np.finfo(np.float64).eps


def barycentric_matrix_nd(from_axes, to_axes) -> np.ndarray:
    """Tensor-product barycentric matrix on meshgrid(..., indexing='ij')
    grids, rows = targets, columns = sources, with exact zero distances
    replaced by EPS, evaluated as the reference does: one reciprocal of the
    product of all distance, weight and normalisation factors
    (quadrature/_interpolation.py:158-213 for 2D, :255-320 for 3D)."""
    dist, w, nf = [], [], []
    for f, t in zip(from_axes, to_axes):
        f = np.asarray(f, dtype=np.float64)
        t = np.asarray(t, dtype=np.float64)
        diff = f[:, None] - f[None, :]
        np.fill_diagonal(diff, 1.0)
        wa = np.prod(diff, axis=0)
        d = t[None, :] - f[:, None]
        d = np.where(d == 0, _EPS, d)
        dist.append(d)
        w.append(wa)
        nf.append(np.sum(1.0 / (wa[:, None] * d), axis=0))
    if len(from_axes) == 2:
        M = 1.0 / (dist[0].T[:, None, :, None] * dist[1].T[None, :, None, :] * w[0][None, None, :, None]
                   * w[1][None, None, None, :] * nf[0][:, None, None, None] * nf[1][None, :, None, None])
        return M.reshape(len(to_axes[0]) * len(to_axes[1]), -1)
    M = 1.0 / (dist[0].T[:, None, None, :, None, None] * dist[1].T[None, :, None, None, :, None]
               * dist[2].T[None, None, :, None, None, :] * w[0][None, None, None, :, None, None]
               * w[1][None, None, None, None, :, None] * w[2][None, None, None, None, None, :]
               * nf[0][:, None, None, None, None, None] * nf[1][None, :, None, None, None, None]
               * nf[2][None, None, :, None, None, None])
    return M.reshape(len(to_axes[0]) * len(to_axes[1]) * len(to_axes[2]), -1)


def _first_containing_leaf(pts: np.ndarray, bounds: np.ndarray) -> np.ndarray:
    """Index of the first leaf whose closed box contains each point, 0 when
    none does (argmax of the containment table, _interpolation_methods.py
    :63-76, :180-195)."""
    d = pts.shape[1]
    inside = np.ones((pts.shape[0], bounds.shape[0]), dtype=bool)
    for a in range(d):
        inside &= (pts[:, a, None] >= bounds[None, :, 2 * a]) & (pts[:, a, None] <= bounds[None, :, 2 * a + 1])
    return np.argmax(inside, axis=1)


def oracle_interp_from_hps(bounds: np.ndarray, p: int, f_evals: np.ndarray, axes):
    """interp_from_hps_2D / _3D (_interpolation_methods.py:23-141, :144-266):
    targets from meshgrid(*axes) (default 'xy' indexing), values reshaped to
    (n_x, n_y[, n_z])[+ (n_src,)].  Returns (values, target_pts)."""
    d = len(axes)
    c = chebyshev_points(p)
    grids = np.meshgrid(*axes)
    target = np.stack(grids, axis=d)
    pts = target.reshape(-1, d)
    leaf = _first_containing_leaf(pts, bounds)
    order = ext_first_order_2D(p) if d == 2 else ext_first_order_3D(p)
    f = np.asarray(f_evals)
    multi = f.ndim == 3
    out = np.zeros((pts.shape[0],) + ((f.shape[2],) if multi else ()), dtype=f.dtype)
    for k in range(pts.shape[0]):
        b = bounds[leaf[k]]
        from_axes = [affine_transform(c, (b[2 * a], b[2 * a + 1])) for a in range(d)]
        if d == 2:
            from_axes[1] = np.flip(from_axes[1])
        I = barycentric_matrix_nd(from_axes, [[pts[k, a]] for a in range(d)])[:, order]
        out[k] = (I @ f[leaf[k]])[0]
    shape = tuple(len(a) for a in axes) + ((f.shape[2],) if multi else ())
    return out.reshape(shape), target


def oracle_interp_to_hps(bounds: np.ndarray, samples: np.ndarray, p: int, axes) -> np.ndarray:
    """interp_to_single_Chebyshev_panel_2D / _3D vmapped over the leaves
    (_interpolation_methods.py:269-340): (n_leaves, p^d)."""
    d = len(axes)
    c = chebyshev_points(p)
    order = ext_first_order_2D(p) if d == 2 else ext_first_order_3D(p)
    out = []
    for b in bounds:
        to_axes = [affine_transform(c, (b[2 * a], b[2 * a + 1])) for a in range(d)]
        if d == 2:
            to_axes[1] = np.flip(to_axes[1])
        I = barycentric_matrix_nd(axes, to_axes)[order, :]
        out.append(I @ np.asarray(samples).reshape(-1))
    return np.stack(out)


# ---------------------------------------------------------------------------
# Adaptive 2D (quadtree) DtN build and solve
# (local_solve/_adaptive_2D_DtN.py, merge/_adaptive_2D_DtN.py:24-433 with
#  merge/_utils_adaptive_2D_DtN.py:11-584, down_pass/_adaptive_2D_DtN.py)
# ---------------------------------------------------------------------------


class QuadNode:
    """Quadtree node of the oracle: bounds b = (xmin, xmax, ymin, ymax),
    children SW, SE, NE, NW."""

    def __init__(self, b, depth=0):
        self.b = tuple(float(x) for x in b)
        self.depth = depth
        self.children = []

    def split(self):
        x0, x1, y0, y1 = self.b
        xm, ym = (x0 + x1) / 2, (y0 + y1) / 2
        self.children = [QuadNode(bb, self.depth + 1) for bb in
                         ((x0, xm, y0, ym), (xm, x1, y0, ym), (xm, x1, ym, y1), (x0, xm, ym, y1))]
        return self.children

    def leaves(self):
        if not self.children:
            return [self]
        return [lf for ch in self.children for lf in ch.leaves()]


def oracle_side_leaves_2D(node: QuadNode):
    """Leaves along S (W->E), E (S->N), N (E->W), W (N->S) of the subtree."""
    lv = node.leaves()
    x0, x1, y0, y1 = node.b
    s = sorted([l for l in lv if l.b[2] == y0], key=lambda l: l.b[0])
    e = sorted([l for l in lv if l.b[1] == x1], key=lambda l: l.b[2])
    n = sorted([l for l in lv if l.b[3] == y1], key=lambda l: -l.b[0])
    w = sorted([l for l in lv if l.b[0] == x0], key=lambda l: -l.b[2])
    return s, e, n, w


def _compress_list_2D(l0, l1):
    """Two facing leaf lists, both ordered outside inward: which panels are
    compressed two to one (_find_compression_list_5..8, :11-197)."""
    o0, o1 = [], []
    i0 = i1 = 0
    while i0 < len(l0) and i1 < len(l1):
        s0, s1 = l0[i0].b[1] - l0[i0].b[0], l1[i1].b[1] - l1[i1].b[0]
        if s0 == s1:
            o0.append(False), o1.append(False)
            i0 += 1
            i1 += 1
        elif s0 < s1:
            o0 += [True, True]
            o1.append(False)
            i0 += 2
            i1 += 1
        else:
            o1 += [True, True]
            o0.append(False)
            i1 += 2
            i0 += 1
    return o0, o1


def _compress2(T, L, flags, axis):
    """_compress_rows_from_lst / _compress_cols_from_lst (:520-584)."""
    q = L.shape[0] if axis == 0 else L.shape[1]
    out, i = [], 0
    while i < len(flags):
        if flags[i] and flags[i + 1]:
            out.append(L @ T[q * i:q * (i + 2)] if axis == 0 else T[:, q * i:q * (i + 2)] @ L)
            i += 2
        else:
            out.append(T[q * i:q * (i + 1)] if axis == 0 else T[:, q * i:q * (i + 1)])
            i += 1
    return np.concatenate(out, axis=axis)


def oracle_adaptive_quad_merge(node: QuadNode, q: int, L_2f1, L_1f2):
    """_adaptive_quad_merge_2D_DtN (merge/_adaptive_2D_DtN.py:198-433)."""
    a, b, c, d = node.children
    sl = [oracle_side_leaves_2D(k) for k in node.children]
    # compression lists, outside inward: a5, b5, b6, c6, c7, d7, d8, a8
    a5, b5 = _compress_list_2D(sl[0][1], sl[1][3][::-1])
    b6, c6 = _compress_list_2D(sl[1][2], sl[2][0][::-1])
    c7, d7 = _compress_list_2D(sl[2][3], sl[3][1][::-1])
    d8, a8 = _compress_list_2D(sl[3][0], sl[0][2][::-1])

    def blocks(k, sets, flags):
        T, h = k.T, k.h
        out = {}
        for i, (ri, fi) in enumerate(zip(sets, flags)):
            for j, (ci, fj) in enumerate(zip(sets, flags)):
                M = T[np.ix_(ri, ci)]
                M = _compress2(M, L_1f2, fi, 0)
                M = _compress2(M, L_2f1, fj, 1)
                out[(i, j)] = M
            out[("h", i)] = _compress2(h[ri], L_1f2, fi, 0)
        return out

    def idx(k):
        n = k.n
        return np.arange(sum(n)), n

    ia, na = idx(a)
    ib, nb = idx(b)
    ic, nc = idx(c)
    id_, nd = idx(d)
    A_ = blocks(a, [np.concatenate([ia[-na[3]:], ia[:na[0]]]), ia[na[0]:na[0] + na[1]],
                    np.flipud(ia[na[0] + na[1]:na[0] + na[1] + na[2]])],
                [[False] * ((na[3] + na[0]) // q), a5, a8])
    B_ = blocks(b, [ib[:nb[0] + nb[1]], ib[nb[0] + nb[1]:nb[0] + nb[1] + nb[2]], np.flipud(ib[-nb[3]:])],
                [[False] * ((nb[0] + nb[1]) // q), b6, b5])
    C_ = blocks(c, [np.flipud(ic[:nc[0]]), ic[nc[0]:nc[0] + nc[1] + nc[2]], ic[-nc[3]:]],
                [c6, [False] * ((nc[1] + nc[2]) // q), c7])
    D_ = blocks(d, [id_[:nd[0]], np.flipud(id_[nd[0]:nd[0] + nd[1]]), id_[nd[0] + nd[1]:]],
                [d8, d7, [False] * ((nd[2] + nd[3]) // q)])
    # a: (1, 5, 8) = (0, 1, 2); b: (2, 6, 5); c: (6, 3, 7); d: (8, 7, 4)
    n1, n5, n8 = A_[(0, 0)].shape[0], A_[(1, 1)].shape[0], A_[(2, 2)].shape[0]
    n2, n6 = B_[(0, 0)].shape[0], B_[(1, 1)].shape[0]
    n3, n7 = C_[(1, 1)].shape[0], C_[(2, 2)].shape[0]
    n4 = D_[(2, 2)].shape[0]
    Z = np.zeros
    Bm = np.block([[A_[(0, 1)], Z((n1, n6)), Z((n1, n7)), A_[(0, 2)]],
                   [B_[(0, 2)], B_[(0, 1)], Z((n2, n7)), Z((n2, n8))],
                   [Z((n3, n5)), C_[(1, 0)], C_[(1, 2)], Z((n3, n8))],
                   [Z((n4, n5)), Z((n4, n6)), D_[(2, 1)], D_[(2, 0)]]])
    Cm = np.block([[A_[(1, 0)], B_[(2, 0)], Z((n5, n3)), Z((n5, n4))],
                   [Z((n6, n1)), B_[(1, 0)], C_[(0, 1)], Z((n6, n4))],
                   [Z((n7, n1)), Z((n7, n2)), C_[(2, 1)], D_[(1, 2)]],
                   [A_[(2, 0)], Z((n8, n2)), Z((n8, n3)), D_[(0, 2)]]])
    Dm = np.block([[A_[(1, 1)] + B_[(2, 2)], B_[(2, 1)], Z((n5, n7)), A_[(1, 2)]],
                   [B_[(1, 2)], B_[(1, 1)] + C_[(0, 0)], C_[(0, 2)], Z((n6, n8))],
                   [Z((n7, n5)), C_[(2, 0)], C_[(2, 2)] + D_[(1, 1)], D_[(1, 0)]],
                   [A_[(2, 1)], Z((n8, n6)), D_[(0, 1)], D_[(0, 0)] + A_[(2, 2)]]])
    A = np.zeros((n1 + n2 + n3 + n4,) * 2)
    o = np.cumsum([0, n1, n2, n3, n4])
    for k, blk in enumerate([A_[(0, 0)], B_[(0, 0)], C_[(1, 1)], D_[(2, 2)]]):
        A[o[k]:o[k + 1], o[k]:o[k + 1]] = blk
    dh = np.concatenate([A_[("h", 1)] + B_[("h", 2)], B_[("h", 1)] + C_[("h", 0)], C_[("h", 2)] + D_[("h", 1)],
                         D_[("h", 0)] + A_[("h", 2)]])
    hx = np.concatenate([A_[("h", 0)], B_[("h", 0)], C_[("h", 1)], D_[("h", 2)]])
    Dinv = np.linalg.inv(Dm)
    S = -Dinv @ Cm
    T = A + Bm @ S
    gt = -Dinv @ dh
    h_out = hx + Bm @ gt
    r = na[3]
    S = np.roll(S, -r, axis=1)
    T = np.roll(np.roll(T, -r, axis=0), -r, axis=1)
    h_out = np.roll(h_out, -r, axis=0)
    flags = dict(a5=a5, b5=b5, b6=b6, c6=c6, c7=c7, d7=d7, d8=d8, a8=a8)
    return S, T, h_out, gt, flags, (n5, n6, n7, n8)


def oracle_adaptive_build_2D(root: QuadNode, p: int, q: int, coeffs: dict, source):
    """Leaf stage with per-leaf rescaled operators, Q / h and h / h, then
    merges from the deepest level up (merge_stage_adaptive_2D_DtN)."""
    leaves = root.leaves()
    dx, dy, dxx, dyy, dxy = diff_operators_2D(p, 1.0)
    ops = {"D_xx": dxx, "D_xy": dxy, "D_yy": dyy, "D_x": dx, "D_y": dy, "I": np.eye(p * p)}
    order = {"D_xx": 2, "D_xy": 2, "D_yy": 2, "D_x": 1, "D_y": 1, "I": 0}
    P = P_2D_DtN(p, q)
    Q = Q_2D_DtN(p, q, dx, dy)
    src = np.asarray(source)
    src = src if src.ndim == 3 else src[..., None]
    for i, lf in enumerate(leaves):
        h = (lf.b[1] - lf.b[0]) / 2
        A = sum(np.asarray(coeffs[k])[i][:, None] * ops[k] / h ** order[k] for k in coeffs if coeffs[k] is not None)
        Y, T, v, hv = leaf_dtn(A[None], src[i:i + 1], P, Q / h)
        lf.Y, lf.T, lf.v, lf.h = Y[0], T[0], v[0], hv[0]
        lf.n = [q, q, q, q]
    gq = gauss_points(q)
    L_2f1 = barycentric_matrix_1D(gq, np.concatenate([affine_transform(gq, (-1.0, 0.0)),
                                                      affine_transform(gq, (0.0, 1.0))]))
    L_1f2 = barycentric_matrix_1D(np.concatenate([affine_transform(gq, (-1.0, 0.0)),
                                                  affine_transform(gq, (0.0, 1.0))]), gq)

    def merge(node):
        for ch in node.children:
            if ch.children:
                merge(ch)
        node.S, node.T, node.h, node.gt, node.flags, node.isz = oracle_adaptive_quad_merge(node, q, L_2f1, L_1f2)
        sl = oracle_side_leaves_2D(node)
        node.n = [q * len(x) for x in sl]

    merge(root)
    root.L_2f1 = L_2f1
    return root


def _expand2(g, L, flags, q):
    out, i, k = [], 0, 0
    while i < len(flags):
        seg = g[k:k + q]
        if flags[i]:
            out.append(L @ seg)
            i += 2
        else:
            out.append(seg)
            i += 1
        k += q
    return np.concatenate(out, axis=0)


def oracle_adaptive_solve_2D(root: QuadNode, bdry, q: int):
    """Down pass (down_pass/_adaptive_2D_DtN.py): every node's interface
    values from S g + g~, decompressed with L_2f1 where the merge compressed,
    then each child's boundary in its own S, E, N, W order; leaves u = Y g + v."""
    L = root.L_2f1
    g0 = np.asarray(bdry)
    g0 = g0 if g0.ndim == 2 else g0[:, None]

    def down(node, g):
        if not node.children:
            node.u = node.Y @ g + node.v
            return
        gi = node.S @ g + node.gt
        n5, n6, n7, n8 = node.isz
        o = np.cumsum([0, n5, n6, n7, n8])
        f = node.flags
        i5, i6, i7, i8 = (gi[o[k]:o[k + 1]] for k in range(4))
        # outside-inward interface values per child side, expanded
        a5, b5 = _expand2(i5, L, f["a5"], q), _expand2(i5, L, f["b5"], q)
        b6, c6 = _expand2(i6, L, f["b6"], q), _expand2(i6, L, f["c6"], q)
        c7, d7 = _expand2(i7, L, f["c7"], q), _expand2(i7, L, f["d7"], q)
        d8, a8 = _expand2(i8, L, f["d8"], q), _expand2(i8, L, f["a8"], q)
        a, b, c, d = node.children
        # merged exterior [a_S, b_S, b_E, c_E, c_N, d_N, d_W, a_W]
        sizes = [a.n[0], b.n[0], b.n[1], c.n[1], c.n[2], d.n[2], d.n[3], a.n[3]]
        e = np.split(g, np.cumsum(sizes)[:-1])
        down(a, np.concatenate([e[0], a5, a8[::-1], e[7]]))
        down(b, np.concatenate([e[1], e[2], b6, b5[::-1]]))
        down(c, np.concatenate([c6[::-1], e[3], e[4], c7]))
        down(d, np.concatenate([d8, d7[::-1], e[5], e[6]]))

    down(root, g0)
    return np.stack([lf.u for lf in root.leaves()])


def L_4f1_2D(p: int) -> np.ndarray:
    """Dense node -> four children interpolation, row blocks a..d each in
    exterior-first order, columns exterior-first (_precompute_operators_2D.py
    :303-328); y runs north to south on the leaf grids."""
    c = chebyshev_points(p)
    lo, hi = affine_transform(c, (-1.0, 0.0)), affine_transform(c, (0.0, 1.0))
    Bl, Bh = barycentric_matrix_1D(c, lo), barycentric_matrix_1D(c, hi)
    r = ext_first_order_2D(p)
    blocks = []
    for bx, by in ((0, 0), (1, 0), (1, 1), (0, 1)):
        Bx = Bh if bx else Bl
        By = (Bh if by else Bl)[::-1, ::-1]
        M = np.kron(Bx, By)
        blocks.append(M[r][:, r])
    return np.concatenate(blocks)


def oracle_adaptive_mesh_2D(root: QuadNode, f, tol: float, p: int, restrict: bool = True, l2: bool = False):
    """generate_adaptive_mesh_level_restriction_2D (_adaptive_discretization_2D.py
    :34-197) with the dense L_4f1 check; ``f`` takes (..., 2) NumPy points.
    Refines in place; returns the number of rounds."""
    Lop = L_4f1_2D(p)
    r = ext_first_order_2D(p)

    def sq_l2(vals, b):
        w = np.outer(chebyshev_weights(p, b[0:2]), chebyshev_weights(p, b[2:4])).ravel()[r]
        return float(np.sum(w * vals ** 2))

    def kids(b):
        return np.array(quad_children_bounds(b))

    if l2:
        root.split()
        gn = sum(sq_l2(f(leaf_points_2D(np.array([lf.b]), p)[0]), lf.b) for lf in root.leaves())
        tol = tol ** 2
    else:
        gn = float(np.max(f(leaf_points_2D(kids(root.b), p).reshape(-1, 2))))

    def find_or_add(node, vol):
        xmin, xmax, ymin, ymax = vol
        side = node.b[1] - node.b[0]
        req = xmax - xmin
        if np.allclose(req * 2, side):
            if not node.children:
                node.split()
                return node
            return None
        xm, ym = (node.b[0] + node.b[1]) / 2, (node.b[2] + node.b[3]) / 2
        i = (0 if ymin < ym else 3) if xmin < xm else (1 if ymin < ym else 2)
        child = node.children[i]
        if np.allclose(side, 4 * req):
            if not child.children:
                child.split()
                return child
            return None
        if side < 2 * req:
            raise ValueError("Requested volume is too large for the current node")
        return find_or_add(child, vol)

    def neighbours(n):
        s = n.b[1] - n.b[0]
        x0, x1, y0, y1 = n.b
        v = []
        if x0 - s >= root.b[0]:
            v.append((x0 - s, x0, y0, y1))
        if x1 + s <= root.b[1]:
            v.append((x1, x1 + s, y0, y1))
        if y0 - s >= root.b[2]:
            v.append((x0, x1, y0 - s, y0))
        if y1 + s <= root.b[3]:
            v.append((x0, x1, y1, y1 + s))
        return v

    queue = root.leaves()
    rounds = 0
    while queue:
        rounds += 1
        ok, nrms = [], []
        for node in queue:
            f0 = f(leaf_points_2D(np.array([node.b]), p)[0])
            kb = kids(node.b)
            f1 = f(leaf_points_2D(kb, p).reshape(-1, 2))
            d = Lop @ f0 - f1
            if l2:
                err = sum(sq_l2(d[k * p * p:(k + 1) * p * p], kb[k]) for k in range(4))
                ok.append(err / gn < tol)
                nrms.append(0.0)
            else:
                nrm = max(gn, float(np.max(np.abs(f1))))
                ok.append(float(np.max(np.abs(d))) / nrm < tol)
                nrms.append(nrm)
        if not l2:
            gn = max(nrms)
        new_queue = []
        for node, good in zip(queue, ok):
            if good:
                continue
            node.split()
            new_queue += node.children
            if restrict:
                pending = [node]
                while pending:
                    fc = pending.pop()
                    for vol in neighbours(fc):
                        n = find_or_add(root, vol)
                        if n is not None:
                            pending.append(n)
                            new_queue += n.children
        queue = new_queue
    return rounds

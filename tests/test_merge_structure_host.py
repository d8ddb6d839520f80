"""Host logic behind the structured merges: the block rectangles of C and B
(2D DtN, ItI, 3D oct merges) against brute-force nonzero patterns, the
two-colour order of the ItI interface matrix and the half-size inverse
formula, and the index conventions of the ItI residual kernel restated in
NumPy against the dense operators G, QH, P, A."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300._index_maps import (colour_perm, merge_rects, oct_merge_maps_dtn, quad_merge_maps_dtn,
                                      quad_merge_maps_iti)
from jaxhps_gb300._refinement import _domain_constants


@pytest.mark.parametrize("kind,size", [("dtn", 1), ("dtn", 3), ("dtn", 14), ("dtn", 56), ("iti", 1), ("iti", 3),
                                       ("iti", 14), ("iti", 28), ("oct", 1), ("oct", 4), ("oct", 16), ("oct", 64)])
def test_merge_rects_cover_exactly_the_nonzero_blocks(kind, size):
    mp, iti = {"dtn": (quad_merge_maps_dtn, False), "iti": (quad_merge_maps_iti, True),
               "oct": (oct_merge_maps_dtn, False)}[kind]
    mp = mp(size)
    c_rects, b_rects = merge_rects(mp, iti)
    n_int, n_ext = mp.n_int, mp.n_ext
    Cm = np.zeros((n_int, n_ext), bool)
    Bm = np.zeros((n_ext, n_int), bool)
    for i in range(n_int):
        cs = {mp.int_c[i, 1]} if iti else {mp.int_c[i, 0], mp.int_c[i, 1]}
        bs = {mp.int_c[i, 0]} if iti else {mp.int_c[i, 0], mp.int_c[i, 1]}
        Cm[i] = np.isin(mp.ext_c, list(cs))
        Bm[:, i] = np.isin(mp.ext_c, list(bs))
    Cr = np.zeros_like(Cm)
    Br = np.zeros_like(Bm)
    seen_c, seen_b = set(), set()
    for i0, li, e0, le, first in c_rects:
        Cr[i0:i0 + li, e0:e0 + le] = True
        assert first == (e0 not in seen_c)
        seen_c.add(e0)
    for e0, le, i0, li, first in b_rects:
        Br[e0:e0 + le, i0:i0 + li] = True
        assert first == (e0 not in seen_b)
        seen_b.add(e0)
    assert np.array_equal(Cr, Cm) and np.array_equal(Br, Bm)


@pytest.mark.parametrize("nc", [1, 3, 8])
def test_two_colour_inverse_of_the_iti_merge_matrix(nc):
    mp = quad_merge_maps_iti(nc)
    cp = colour_perm(mp)
    assert cp is not None and len(cp) == mp.n_int
    rng = np.random.default_rng(0)
    R = rng.standard_normal((4, 4 * nc, 4 * nc)) + 1j * rng.standard_normal((4, 4 * nc, 4 * nc))
    ni = mp.n_int
    D = np.eye(ni, dtype=complex)
    for u in range(ni):
        pc, pl = mp.int_c[u, 1], mp.int_l[u, 1]
        for w in range(ni):
            if mp.int_c[w, 0] == pc:
                D[u, w] += 0.3 * R[pc, pl, mp.int_l[w, 0]]
    Dp = D[np.ix_(cp, cp)]
    h = ni // 2
    assert np.allclose(Dp[:h, :h], np.eye(h)) and np.allclose(Dp[h:, h:], np.eye(h))
    D12, D21 = Dp[:h, h:], Dp[h:, :h]
    Wi = np.linalg.inv(np.eye(h) - D12 @ D21)
    Dinv = np.empty_like(D)
    Dinv[np.ix_(cp, cp)] = np.block([[Wi, -Wi @ D12], [-D21 @ Wi, np.eye(h) + D21 @ Wi @ D12]])
    assert np.allclose(Dinv, np.linalg.inv(D))


def test_iti_residual_index_conventions():
    """The residual kernel's point / side conventions (perm, side t-th point,
    outward normal derivative per side, P on p-1 points per side, Q on p) on
    the dense operators of PDEProblem."""
    p, q, eta = 7, 5, 3.0
    dom = hps.Domain(p=p, q=q, root=hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0), L=1)
    x = dom.interior_points
    rng = np.random.default_rng(0)
    cxx = 1 + 0.1 * rng.standard_normal(x.shape[:2])
    cxy = rng.standard_normal(x.shape[:2])
    ci = rng.standard_normal(x.shape[:2]) + 1j * rng.standard_normal(x.shape[:2])
    pde = hps.PDEProblem(dom, source=np.zeros(x.shape[:2]), D_xx_coefficients=cxx, D_xy_coefficients=cxy,
                         D_yy_coefficients=cxx, I_coefficients=ci, use_ItI=True, eta=eta)
    c = {k: v.numpy() for k, v in _domain_constants(dom, torch.device("cpu")).items()}
    nl, pp = x.shape[:2]
    m, ncb, nq = p - 1, 4 * (p - 1), 4 * q
    u = rng.standard_normal((nl, pp)) + 1j * rng.standard_normal((nl, pp))
    t = rng.standard_normal((nl, nq)) + 1j * rng.standard_normal((nl, nq))
    D1, D2, Ps, Qs, perm, ih = c["D1"], c["D2"], c["Pside"], c["Qside"], c["perm"], c["inv_half"][0]
    for leaf in range(nl):
        A = np.diag(cxx[leaf]) @ (pde.D_xx + pde.D_yy) + np.diag(cxy[leaf]) @ pde.D_xy + np.diag(ci[leaf])
        U = np.zeros(pp, complex)
        U[perm] = u[leaf]
        Ug = U.reshape(p, p)                                   # [ix, iy], iy = 0 the north row
        uxx = ih * ih * D2 @ Ug
        uyy = ih * ih * Ug @ D2.T
        uy = -ih * Ug @ D1.T
        uxy = ih * D1 @ uy
        Au = (cxx[leaf] * (uxx + uyy).ravel()[perm] + cxy[leaf] * uxy.ravel()[perm] + ci[leaf] * U[perm])
        assert np.allclose(Au[ncb:], (A @ u[leaf])[ncb:])
        nd = np.stack([ih * Ug[:, :] @ D1[p - 1], ih * (D1[p - 1] @ Ug)[::-1], -ih * (Ug @ D1[0])[::-1],
                       -ih * (D1[0] @ Ug)])       # S, E, N, W outward derivatives along each side
        side_pt = lambda s, k: perm[(s * m + k) % ncb]   # noqa: E731
        G = np.array([nd[k // m, k % m] + 1j * eta * U[side_pt(k // m, k % m)] for k in range(ncb)])
        Pt = np.array([Ps[k % m] @ t[leaf, (k // m) * q:(k // m + 1) * q] for k in range(ncb)])
        assert np.allclose(G, pde.G @ u[leaf]) and np.allclose(Pt, pde.P @ t[leaf])
        to = np.array([Qs[k % q] @ np.array([nd[k // q, s] - 1j * eta * U[side_pt(k // q, s)] for s in range(p)])
                       for k in range(nq)])
        assert np.allclose(to, pde.QH @ u[leaf])

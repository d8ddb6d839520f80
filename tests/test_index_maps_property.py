"""Property tests (hypothesis) of the merge index maps: for random interface
sizes and random child operators, the gather + Schur complement that the
maps drive (emulated in NumPy, as hps_merge_level_dtn computes it)
reproduces the oracle's quad and oct merges, and the down-pass code map
reproduces the oracle's down propagation.  Skipped where hypothesis is not
installed."""

import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as hs  # noqa: E402

from jaxhps_gb300 import _index_maps as im  # noqa: E402
from oracle import hps_oracle as O  # noqa: E402


def _merge_by_maps(Ts, hs_, maps):
    Tm, hm = np.stack(Ts), np.stack(hs_)
    ni, ne = maps.n_int, maps.n_ext
    D = np.zeros((ni, ni))
    for t in range(2):
        c, l = maps.int_c[:, t], maps.int_l[:, t]
        lj = maps.loc[c]                               # (ni, ni): local index of interface j in child c
        ok = lj >= 0
        rows = Tm[c[:, None], l[:, None], np.where(ok, lj, 0)]
        D += np.where(ok, rows, 0.0)
    ec, el = maps.ext_c, maps.ext_l
    li = maps.loc[ec].T                                # (ni, ne)
    okc = li >= 0
    C = np.where(okc, Tm[ec[None, :], np.where(okc, li, 0), el[None, :]], 0.0)
    B = np.where(okc.T, Tm[ec[:, None], el[:, None], np.where(okc, li, 0).T], 0.0)
    same = ec[:, None] == ec[None, :]
    A = np.where(same, Tm[ec[:, None], el[:, None], el[None, :]], 0.0)
    dh = hm[maps.int_c[:, 0], maps.int_l[:, 0]] + hm[maps.int_c[:, 1], maps.int_l[:, 1]]
    S = -np.linalg.solve(D, C)
    gt = -np.linalg.solve(D, dh)
    return S, A + B @ S, hm[ec, el] + B @ gt, gt


def _children(rng, k, n, ns=2):
    Ts = [rng.standard_normal((n, n)) + 3 * np.sqrt(n) * np.eye(n) for _ in range(k)]
    hs_ = [rng.standard_normal((n, ns)) for _ in range(k)]
    return Ts, hs_


@settings(max_examples=25, deadline=None)
@given(nc=hs.integers(1, 12), seed=hs.integers(0, 2 ** 31 - 1))
def test_quad_maps_reproduce_oracle_merge(nc, seed):
    Ts, hs_ = _children(np.random.default_rng(seed), 4, 4 * nc)
    S, T, h, gt = O.quad_merge_dtn(*Ts, *hs_)
    S2, T2, h2, gt2 = _merge_by_maps(Ts, hs_, im.quad_merge_maps_dtn(nc))
    for a, b in ((S, S2), (T, T2), (h, h2), (gt, gt2)):
        assert np.allclose(a, b, rtol=1e-9, atol=1e-9)


@settings(max_examples=10, deadline=None)
@given(q=hs.integers(1, 4), seed=hs.integers(0, 2 ** 31 - 1))
def test_oct_maps_reproduce_oracle_merge(q, seed):
    nf = q * q
    Ts, hs_ = _children(np.random.default_rng(seed), 8, 6 * nf)
    S, T, h, gt = O.oct_merge_dtn(Ts, hs_)
    S2, T2, h2, gt2 = _merge_by_maps(Ts, hs_, im.oct_merge_maps_dtn(nf))
    for a, b in ((S, S2), (T, T2), (h, h2), (gt, gt2)):
        assert np.allclose(a, b, rtol=1e-9, atol=1e-9)


@settings(max_examples=25, deadline=None)
@given(nc=hs.integers(1, 12), ns=hs.integers(1, 4), seed=hs.integers(0, 2 ** 31 - 1))
def test_quad_code_map_reproduces_oracle_down_pass(nc, ns, seed):
    rng = np.random.default_rng(seed)
    S = rng.standard_normal((4 * nc, 8 * nc))
    g = rng.standard_normal((8 * nc, ns))
    gt = rng.standard_normal((4 * nc, ns))
    ref = O._propagate_down_dtn(S, g, gt)
    maps = im.quad_merge_maps_dtn(nc)
    gi = S @ g + gt
    full = np.concatenate([g, gi])                     # exterior first, then interfaces
    idx = np.where(maps.code >= 0, maps.code, 8 * nc - maps.code - 1)
    assert np.allclose(full[idx], ref)

"""Host-side index maps that drive the merge gather and down-pass scatter
kernels.

A merge of ``nch`` children, each with ``nb`` boundary points, is described
by one integer ``code`` per (child, local boundary point):
``code >= 0`` is the point's index in the merged node's exterior (in the
final, already rolled order), ``code < 0`` is interface unknown
``-(code+1)``.  From ``code`` the DtN gather maps are derived: the two
(child, local) copies of every interface point, the (child, local) of every
exterior point, and a child x interface table of local indices.
"""

from __future__ import annotations

from dataclasses import dataclass
from functools import lru_cache

import numpy as np
import torch


# Code of a padding slot (a child with fewer boundary points than the merge's
# common child size); the C ABI's HPS_CODE_PAD.
CODE_PAD = -(2 ** 31)


@dataclass
class MergeMaps:
    nch: int
    nb: int
    n_int: int
    n_ext: int
    code: np.ndarray    # (nch, nb)
    int_c: np.ndarray   # (n_int, 2)
    int_l: np.ndarray   # (n_int, 2)
    ext_c: np.ndarray   # (n_ext,)
    ext_l: np.ndarray   # (n_ext,)
    loc: np.ndarray     # (nch, n_int)

    def device(self, dev):
        key = str(dev)
        cache = self.__dict__.setdefault("_dev", {})
        if key not in cache:
            def t(a):
                return torch.as_tensor(np.ascontiguousarray(a, dtype=np.int32), device=dev)
            cache[key] = {k: t(getattr(self, k)) for k in ("code", "int_c", "int_l", "ext_c", "ext_l", "loc")}
        return cache[key]


def maps_from_code(code: np.ndarray, n_ext: int, n_int: int) -> MergeMaps:
    nch, nb = code.shape
    int_c = np.full((n_int, 2), -1, dtype=np.int64)
    int_l = np.full((n_int, 2), -1, dtype=np.int64)
    ext_c = np.full(n_ext, -1, dtype=np.int64)
    ext_l = np.full(n_ext, -1, dtype=np.int64)
    loc = np.full((nch, n_int), -1, dtype=np.int64)
    fill = np.zeros(n_int, dtype=np.int64)
    for c in range(nch):
        for k in range(nb):
            cd = code[c, k]
            if cd == CODE_PAD:
                continue
            if cd >= 0:
                assert ext_c[cd] < 0, "exterior point mapped twice"
                ext_c[cd], ext_l[cd] = c, k
            else:
                i = -cd - 1
                assert fill[i] < 2, "interface point shared by more than two children"
                int_c[i, fill[i]], int_l[i, fill[i]] = c, k
                fill[i] += 1
                loc[c, i] = k
    assert (ext_c >= 0).all(), "exterior point not covered"
    assert (fill == 2).all(), "interface point without two sides"
    return MergeMaps(nch, nb, n_int, n_ext, code, int_c, int_l, ext_c, ext_l, loc)


def _runs(keys):
    """Maximal runs [start, start+len) of equal consecutive keys."""
    out, i, n = [], 0, len(keys)
    while i < n:
        j = i + 1
        while j < n and keys[j] == keys[i]:
            j += 1
        out.append((i, j - i, keys[i]))
        i = j
    return out


def merge_rects(maps, iti: bool):
    """Block structure of a merge's C (n_int x n_ext) and B (n_ext x n_int).

    Row i of C holds the partner child's (ItI) or both children's (DtN)
    exterior entries, column j of B its owner's (ItI) or both children's; all
    else is zero.  Returns int32 arrays (n, 5) of rectangles
    (i0, n_i, e0, n_e, first) for C and (e0, n_e, i0, n_i, first) for B, as
    hps_merge_args takes them, or None when they would not save a fifth of
    the dense products.  Cached on the maps object."""
    cache = maps.__dict__.setdefault("_rects", {})
    if iti in cache:
        return cache[iti]
    int_c = np.asarray(maps.int_c)
    if iti:
        cset = [frozenset((int(c),)) for c in int_c[:, 1]]
        bset = [frozenset((int(c),)) for c in int_c[:, 0]]
    else:
        cset = bset = [frozenset((int(a), int(b))) for a, b in int_c]
    ext_runs = _runs([int(c) for c in maps.ext_c])
    c_rects, b_rects = [], []
    seen = set()
    for e0, le, ch in ext_runs:
        for i0, li, cs in _runs(cset):
            if ch in cs:
                c_rects.append((i0, li, e0, le, 0 if e0 in seen else 1))
                seen.add(e0)
    seen = set()
    for e0, le, ch in ext_runs:
        for i0, li, bs in _runs(bset):
            if ch in bs:
                b_rects.append((e0, le, i0, li, 0 if e0 in seen else 1))
                seen.add(e0)
    covered_c = {r[2] for r in c_rects}
    covered_b = {r[0] for r in b_rects}
    all_e = {e0 for e0, _, _ in ext_runs}
    out = None
    work = sum(r[1] * r[3] for r in c_rects) + sum(r[1] * r[3] for r in b_rects)
    if covered_c == all_e and covered_b == all_e and work <= 0.8 * 2 * maps.n_int * maps.n_ext:
        out = (np.ascontiguousarray(np.array(c_rects, dtype=np.int32)),
               np.ascontiguousarray(np.array(b_rects, dtype=np.int32)))
    cache[iti] = out
    return out


def colour_perm(maps):
    """Two-colouring of an ItI merge's interface unknowns, or None.

    Unknown u (owned by child own(u), its equation coupling to the partner
    child par(u)) gets the colour of its owner.  When the children split in
    two classes with every owner/partner pair across them and the classes
    hold n_int/2 unknowns each, D = [[I, D12], [D21, I]] in the order
    returned (colour X first) and its inverse needs only the n_int/2 inverse
    of I - D12 D21 (hps_merge_args.n_x, colour_perm).  Cached on the maps."""
    cache = maps.__dict__.setdefault("_colour", {})
    if "perm" in cache:
        return cache["perm"]
    own = np.asarray(maps.int_c)[:, 0]
    par = np.asarray(maps.int_c)[:, 1]
    col = {}
    edges = {}
    for a, b in zip(own.tolist(), par.tolist()):
        edges.setdefault(a, set()).add(b)
        edges.setdefault(b, set()).add(a)
    ok = True
    for start in sorted(edges):
        if start in col:
            continue
        col[start] = 0
        stack = [start]
        while stack and ok:
            c = stack.pop()
            for d in edges[c]:
                if d not in col:
                    col[d] = 1 - col[c]
                    stack.append(d)
                elif col[d] == col[c]:
                    ok = False
    out = None
    if ok:
        cu = np.array([col[int(c)] for c in own])
        x, y = np.nonzero(cu == 0)[0], np.nonzero(cu == 1)[0]
        if len(x) == len(y) == maps.n_int // 2 and 2 * len(x) == maps.n_int:
            out = np.ascontiguousarray(np.concatenate([x, y]).astype(np.int32))
    cache["perm"] = out
    return out


@lru_cache(maxsize=None)
def quad_merge_maps_dtn(nc: int) -> MergeMaps:
    """2D quad merge of children a,b,c,d (SW,SE,NE,NW) with nc Gauss points
    per child side.

    Exterior order after the roll of merge/_uniform_2D_DtN.py:343-346:
    [a_S, b_S, b_E, c_E, c_N, d_N, d_W, a_W].  Interfaces 5 (a|b), 6 (b|c),
    7 (c|d), 8 (d|a) in the orientation of get_quadmerge_blocks_* (:384-437):
    a's and b's own side order for 5 and 6 ... with the partner side flipped.
    """
    nb = 4 * nc
    code = np.zeros((4, nb), dtype=np.int64)
    t = np.arange(nc)
    # exterior
    code[0, 0:nc] = 0 * nc + t            # a_S
    code[1, 0:nc] = 1 * nc + t            # b_S
    code[1, nc:2 * nc] = 2 * nc + t       # b_E
    code[2, nc:2 * nc] = 3 * nc + t       # c_E
    code[2, 2 * nc:3 * nc] = 4 * nc + t   # c_N
    code[3, 2 * nc:3 * nc] = 5 * nc + t   # d_N
    code[3, 3 * nc:4 * nc] = 6 * nc + t   # d_W
    code[0, 3 * nc:4 * nc] = 7 * nc + t   # a_W
    # interfaces (value -(i+1))
    i5, i6, i7, i8 = t, nc + t, 2 * nc + t, 3 * nc + t
    code[0, nc + t] = -(i5 + 1)
    code[1, 4 * nc - 1 - t] = -(i5 + 1)
    code[1, 2 * nc + t] = -(i6 + 1)
    code[2, nc - 1 - t] = -(i6 + 1)
    code[2, 3 * nc + t] = -(i7 + 1)
    code[3, 2 * nc - 1 - t] = -(i7 + 1)
    code[3, t] = -(i8 + 1)
    code[0, 3 * nc - 1 - t] = -(i8 + 1)
    return maps_from_code(code, n_ext=8 * nc, n_int=4 * nc)


@dataclass
class ItiMergeMaps:
    """ItI quad merge: interface unknowns are the children's incoming
    impedances on each side of every interface (8nc of them), ordered
    [a5, b5, b6, c6, c7, d7, d8, a8] as after the row reordering of
    merge/_uniform_2D_ItI.py:360-373.  Unknown u lives at (unk_c, unk_l);
    its equation involves the partner child across the interface
    (par_c, par_l)."""
    nch: int
    nb: int
    n_int: int
    n_ext: int
    code: np.ndarray
    int_c: np.ndarray   # (n_int, 2): [own child, partner child]
    int_l: np.ndarray   # (n_int, 2): [own local, partner local]
    ext_c: np.ndarray
    ext_l: np.ndarray
    loc: np.ndarray     # unused by the ItI gather (kept for a uniform interface)

    device = MergeMaps.device


@lru_cache(maxsize=None)
def quad_merge_maps_iti(nc: int) -> ItiMergeMaps:
    dtn = quad_merge_maps_dtn(nc)
    t = np.arange(nc)
    # (child, local) of each unknown block, in the reference's final order
    blocks = [
        (0, nc + t),               # a5: a's E side
        (1, 4 * nc - 1 - t),       # b5: b's W side, reversed
        (1, 2 * nc + t),           # b6: b's N side
        (2, nc - 1 - t),           # c6: c's S side, reversed
        (2, 3 * nc + t),           # c7: c's W side
        (3, 2 * nc - 1 - t),       # d7: d's E side, reversed
        (3, t),                    # d8: d's S side
        (0, 3 * nc - 1 - t),       # a8: a's N side, reversed
    ]
    partner = [1, 0, 3, 2, 5, 4, 7, 6]
    n_int = 8 * nc
    own_c = np.concatenate([np.full(nc, c) for c, _ in blocks])
    own_l = np.concatenate([l for _, l in blocks])
    par_c = np.concatenate([np.full(nc, blocks[partner[b]][0]) for b in range(8)])
    par_l = np.concatenate([blocks[partner[b]][1] for b in range(8)])
    code = dtn.code.copy()
    for u in range(n_int):
        code[own_c[u], own_l[u]] = -(u + 1)
    return ItiMergeMaps(4, 4 * nc, n_int, 8 * nc, code, np.stack([own_c, par_c], 1), np.stack([own_l, par_l], 1),
                        dtn.ext_c, dtn.ext_l, np.full((4, n_int), -1, dtype=np.int64))


# Octree children a..h as (x, y, z) half bits (_grid_creation_3D.py:28-74).
OCT_CHILD_BITS = ((0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1), (0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0))
# Interfaces in the reference's label order 9..20 (merge/_schur_complement.py:293-774):
# a|b, b|c, c|d, d|a, e|f, f|g, g|h, h|e, a|e, b|f, c|g, d|h.
OCT_INTERFACES = ((0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7))


@lru_cache(maxsize=None)
def oct_merge_maps_dtn(nf: int) -> MergeMaps:
    """3D oct merge of children a..h, each face holding nf Gauss points.

    Child faces are -x, +x, -y, +y, -z, +z (nf points each, same in-face
    order on both sides of an interface, so no flips).  The merged exterior
    is face by face, each face made of the four touching children's faces in
    2D quad order of the face (the re-ordering of
    merge/_uniform_3D_DtN.py:442-541).  Interface i holds the nf points of
    OCT_INTERFACES[i]."""
    from ._grid_creation_3D import FACE_TRAVERSAL

    nb = 6 * nf
    code = np.zeros((8, nb), dtype=np.int64)
    t = np.arange(nf)
    for F in range(6):
        axis, side = F // 2, F % 2
        kids = [c for c in FACE_TRAVERSAL[axis] if OCT_CHILD_BITS[c][axis] == side]
        for j, c in enumerate(kids):
            code[c, F * nf + t] = F * 4 * nf + j * nf + t
    for i, (c0, c1) in enumerate(OCT_INTERFACES):
        axis = next(k for k in range(3) if OCT_CHILD_BITS[c0][k] != OCT_CHILD_BITS[c1][k])
        lo, hi = (c0, c1) if OCT_CHILD_BITS[c0][axis] == 0 else (c1, c0)
        code[lo, (2 * axis + 1) * nf + t] = -(i * nf + t + 1)
        code[hi, (2 * axis) * nf + t] = -(i * nf + t + 1)
    return maps_from_code(code, n_ext=24 * nf, n_int=12 * nf)

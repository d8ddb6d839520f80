"""Level-batched FP64 oracle for the uniform 2D DtN path (TEST INFRASTRUCTURE ONLY).

The same algorithm as ``oracle/hps_oracle.py`` (and therefore as the
reference, meliao/jaxhps), organised the way the reference's ``vmap`` over
all leaves or all merges of a level organises it: every stage works on the
whole level as stacked arrays, so that LAPACK / BLAS see batches and the
host's cores can share them.  It exists to time the reference algorithm on
the CPU at the benchmark's full size (``bench.py``'s CPU baseline and
``--impl reference``) and to give the full-size FP64 solution the GPU result
is compared against.  Only ``tests/`` and ``bench.py`` import it.

Threading: a level with many small problems is split into chunks that run on
a thread pool (NumPy releases the GIL inside LAPACK and BLAS) with OpenBLAS
held at one thread; a level with few large problems runs its calls with
OpenBLAS on every thread.  OpenBLAS's thread count is set through its own
``*_set_num_threads`` entry point found in the loaded library.

Correspondence with the reference (paths relative to the reference root):
  * leaf stage: local_solve/_uniform_2D_DtN.py:182-273 (assemble_diff_operator,
    get_DtN: inv(A_ii), Y = [I; -inv(A_ii) A_ie] P, T = Q Y, v, h = Q v);
  * merge level: merge/_uniform_2D_DtN.py:206-348 (B, C, D blocks of the four
    children, the roll of the merged exterior by -nc) with
    merge/_schur_complement.py:182-237 (S = -D^-1 C, T = B S + A,
    g~ = -D^-1 dh, h = h_ext + B g~);
  * down pass: down_pass/_uniform_2D_DtN.py:125-189 (g_int = S g + g~, the
    children's boundary assembly with the interface flips) and :114-120
    (u = Y g + v).
"""

from __future__ import annotations

import ctypes
import os
from concurrent.futures import ThreadPoolExecutor
from contextlib import contextmanager

import numpy as np

from oracle import hps_oracle as O

# ---------------------------------------------------------------------------
# OpenBLAS thread control
# ---------------------------------------------------------------------------

_SETTERS = ("scipy_openblas_set_num_threads64_", "scipy_openblas_set_num_threads",
            "openblas_set_num_threads64_", "openblas_set_num_threads")
_GETTERS = ("scipy_openblas_get_num_threads64_", "scipy_openblas_get_num_threads",
            "openblas_get_num_threads64_", "openblas_get_num_threads")
_blas = None


def _blas_fns():
    """(setter, getter) of the OpenBLAS loaded by NumPy, or (None, None)."""
    global _blas
    if _blas is not None:
        return _blas
    _blas = (None, None)
    try:
        with open("/proc/self/maps") as fh:
            paths = sorted({ln.split()[-1] for ln in fh if "openblas" in ln.lower() and "/" in ln})
    except OSError:
        paths = []
    for p in paths:
        try:
            lib = ctypes.CDLL(p)
        except OSError:
            continue
        s = next((getattr(lib, n) for n in _SETTERS if hasattr(lib, n)), None)
        g = next((getattr(lib, n) for n in _GETTERS if hasattr(lib, n)), None)
        if s is not None and g is not None:
            s.argtypes, s.restype, g.restype = [ctypes.c_int], None, ctypes.c_int
            _blas = (s, g)
            break
    return _blas


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


@contextmanager
def blas_threads(n: int):
    s, g = _blas_fns()
    if s is None:
        yield False
        return
    old = g()
    s(int(n))
    try:
        yield True
    finally:
        s(old)


class Runner:
    """Runs chunked work on ``threads`` host threads (one BLAS thread each),
    or whole calls with BLAS on all of them."""

    def __init__(self, threads: int | None = None):
        self.threads = max(1, int(threads or host_threads()))
        self.pool = ThreadPoolExecutor(self.threads) if self.threads > 1 else None

    def close(self):
        if self.pool is not None:
            self.pool.shutdown()

    def chunks(self, n: int, min_chunk: int = 1):
        k = max(1, min(n // max(min_chunk, 1), 4 * self.threads))
        edges = np.linspace(0, n, k + 1).astype(int)
        return [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]

    def map(self, fn, n: int, min_chunk: int = 1):
        """fn(lo, hi) over chunks of range(n)."""
        parts = self.chunks(n, min_chunk)
        if self.pool is None or len(parts) == 1:
            with blas_threads(self.threads):
                for lo, hi in parts:
                    fn(lo, hi)
            return
        with blas_threads(1):
            list(self.pool.map(lambda ab: fn(*ab), parts))


# ---------------------------------------------------------------------------
# Leaf stage
# ---------------------------------------------------------------------------


def leaf_stage_dtn(coeffs: dict, ops: dict, source: np.ndarray, P: np.ndarray, Q: np.ndarray, run: Runner):
    """All leaves at once, chunked (get_DtN vmapped, local_solve/_uniform_2D_DtN.py:228-280).
    ``coeffs``: name -> (n_leaves, n_pts) or None; ``source``: (n_leaves, n_pts, nsrc)."""
    n_cb, ng = P.shape
    active = [(np.asarray(coeffs[k]), ops[k]) for k in coeffs if coeffs[k] is not None]
    nl, npts = active[0][0].shape
    ns = source.shape[-1]
    Y = np.empty((nl, npts, ng))
    T = np.empty((nl, ng, ng))
    v = np.zeros((nl, npts, ns))
    h = np.empty((nl, ng, ns))
    Y[:, :n_cb] = P

    def work(lo, hi):
        # interior rows of A = sum_k diag(c_k) D_k (the exterior rows are not used by get_DtN)
        A = np.zeros((hi - lo, npts - n_cb, npts))
        for c, D in active:
            A += c[lo:hi, n_cb:, None] * D[None, n_cb:, :]
        inv = np.linalg.inv(A[:, :, n_cb:])
        L2 = -(inv @ A[:, :, :n_cb])
        Y[lo:hi, n_cb:] = L2 @ P
        v[lo:hi, n_cb:] = inv @ source[lo:hi, n_cb:]
        T[lo:hi] = Q @ Y[lo:hi]
        h[lo:hi] = Q @ v[lo:hi]

    run.map(work, nl, min_chunk=8)
    return Y, T, v, h


# ---------------------------------------------------------------------------
# Merge level
# ---------------------------------------------------------------------------


def _bsub(X, i, j):
    return X[:, i[:, None], j[None, :]]


def _bblock(rows, nb):
    """np.block for a batch: rows of (nb, r, c) blocks or (r, c) zero shapes."""
    out = []
    for row in rows:
        r = next(b.shape[1] for b in row if isinstance(b, np.ndarray))
        parts = [b if isinstance(b, np.ndarray) else np.zeros((nb, r, b[1])) for b in row]
        out.append(np.concatenate(parts, axis=2))
    return np.concatenate(out, axis=1)


def merge_level_dtn(T: np.ndarray, h: np.ndarray, run: Runner):
    """One level of quad merges (merge/_uniform_2D_DtN.py:206-348 with
    merge/_schur_complement.py:182-237), all merges at once.  T: (4m, 4nc, 4nc),
    h: (4m, 4nc, nsrc).  Returns S (m, 4nc, 8nc), T (m, 8nc, 8nc),
    h (m, 8nc, nsrc), g~ (m, 4nc, nsrc)."""
    nm = T.shape[0] // 4
    nc = T.shape[1] // 4
    ns = h.shape[-1]
    (a1, a5, a8), (b2, b6, b5), (c6, c3, c7), (d8, d7, d4) = O._quad_side_indices(nc)
    S_out = np.empty((nm, 4 * nc, 8 * nc))
    T_out = np.empty((nm, 8 * nc, 8 * nc))
    h_out = np.empty((nm, 8 * nc, ns))
    g_out = np.empty((nm, 4 * nc, ns))
    ze, zi, zz = (2 * nc, nc), (nc, 2 * nc), (nc, nc)

    def work(lo, hi):
        nb = hi - lo
        Ta, Tb, Tc, Td = (T[4 * lo + k:4 * hi:4] for k in range(4))
        ha, hb, hc, hd = (h[4 * lo + k:4 * hi:4] for k in range(4))
        B = _bblock([[_bsub(Ta, a1, a5), ze, ze, _bsub(Ta, a1, a8)],
                     [_bsub(Tb, b2, b5), _bsub(Tb, b2, b6), ze, ze],
                     [ze, _bsub(Tc, c3, c6), _bsub(Tc, c3, c7), ze],
                     [ze, ze, _bsub(Td, d4, d7), _bsub(Td, d4, d8)]], nb)
        C = _bblock([[_bsub(Ta, a5, a1), _bsub(Tb, b5, b2), zi, zi],
                     [zi, _bsub(Tb, b6, b2), _bsub(Tc, c6, c3), zi],
                     [zi, zi, _bsub(Tc, c7, c3), _bsub(Td, d7, d4)],
                     [_bsub(Ta, a8, a1), zi, zi, _bsub(Td, d8, d4)]], nb)
        D = _bblock([[_bsub(Ta, a5, a5) + _bsub(Tb, b5, b5), _bsub(Tb, b5, b6), zz, _bsub(Ta, a5, a8)],
                     [_bsub(Tb, b6, b5), _bsub(Tb, b6, b6) + _bsub(Tc, c6, c6), _bsub(Tc, c6, c7), zz],
                     [zz, _bsub(Tc, c7, c6), _bsub(Tc, c7, c7) + _bsub(Td, d7, d7), _bsub(Td, d7, d8)],
                     [_bsub(Ta, a8, a5), zz, _bsub(Td, d8, d7), _bsub(Td, d8, d8) + _bsub(Ta, a8, a8)]], nb)
        dh = np.concatenate([ha[:, a5] + hb[:, b5], hb[:, b6] + hc[:, c6], hc[:, c7] + hd[:, d7],
                             hd[:, d8] + ha[:, a8]], axis=1)
        h_ext = np.concatenate([ha[:, a1], hb[:, b2], hc[:, c3], hd[:, d4]], axis=1)
        Dinv = np.linalg.inv(D)
        S = -(Dinv @ C)
        Tm = B @ S
        for k, (X, e) in enumerate(((Ta, a1), (Tb, b2), (Tc, c3), (Td, d4))):
            sl = slice(2 * nc * k, 2 * nc * (k + 1))
            Tm[:, sl, sl] += _bsub(X, e, e)
        gt = -(Dinv @ dh)
        ho = h_ext + B @ gt
        # the reference rolls the merged exterior by -nc (merge/_uniform_2D_DtN.py:343-346)
        h_out[lo:hi] = np.roll(ho, -nc, axis=1)
        T_out[lo:hi] = np.roll(np.roll(Tm, -nc, axis=1), -nc, axis=2)
        S_out[lo:hi] = np.roll(S, -nc, axis=2)
        g_out[lo:hi] = gt

    if nm >= 2 * run.threads:
        run.map(work, nm)
    else:
        with blas_threads(run.threads):
            work(0, nm)
    return S_out, T_out, h_out, g_out


def merge_stage_dtn(T, h, L: int, run: Runner):
    S_lst, g_lst = [], []
    for _ in range(max(L, 1)):
        S, T, h, g = merge_level_dtn(T, h, run)
        S_lst.append(S)
        g_lst.append(g)
    return S_lst, g_lst, T[0], h[0]


# ---------------------------------------------------------------------------
# Down pass
# ---------------------------------------------------------------------------


def down_pass_dtn(bdry: np.ndarray, S_lst, g_lst, Y, v, run: Runner):
    """bdry (n_bdry, nsrc) -> leaf solutions (n_leaves, n_pts, nsrc)
    (down_pass/_uniform_2D_DtN.py:7-189), level by level."""
    g = bdry[None]
    for lvl in range(len(S_lst) - 1, -1, -1):
        S, gt = S_lst[lvl], g_lst[lvl]
        nm = S.shape[0]
        nc = g.shape[1] // 8
        ns = g.shape[2]
        out = np.empty((nm, 4, 4 * nc, ns))

        def work(lo, hi, S=S, gt=gt, g=g, nc=nc, out=out):
            gg = g[lo:hi]
            gi = S[lo:hi] @ gg + gt[lo:hi]
            g5, g6, g7, g8 = (gi[:, k * nc:(k + 1) * nc] for k in range(4))
            out[lo:hi, 0] = np.concatenate([gg[:, :nc], g5, g8[:, ::-1], gg[:, 7 * nc:]], axis=1)
            out[lo:hi, 1] = np.concatenate([gg[:, nc:3 * nc], g6, g5[:, ::-1]], axis=1)
            out[lo:hi, 2] = np.concatenate([g6[:, ::-1], gg[:, 3 * nc:5 * nc], g7], axis=1)
            out[lo:hi, 3] = np.concatenate([g8, g7[:, ::-1], gg[:, 5 * nc:7 * nc]], axis=1)

        if nm >= 2 * run.threads:
            run.map(work, nm)
        else:
            with blas_threads(run.threads):
                work(0, nm)
        g = out.reshape(4 * nm, 4 * nc, ns)
    nl = Y.shape[0]
    u = np.empty((nl, Y.shape[1], g.shape[2]))

    def leaves(lo, hi):
        u[lo:hi] = Y[lo:hi] @ g[lo:hi] + v[lo:hi]

    run.map(leaves, nl, min_chunk=64)
    return u


# ---------------------------------------------------------------------------
# Whole problem
# ---------------------------------------------------------------------------


class LevelProblem2D:
    """Uniform 2D DtN build + solve with level-batched stages; the arguments
    and results of ``hps_oracle.Problem2D`` (DtN)."""

    def __init__(self, root_bounds, L, p, q, coeffs, source, threads=None):
        self.base = O.Problem2D(root_bounds, L, p, q, {k: None for k in O.Problem2D.OPS}, np.zeros((1, 1)))
        self.base.coeffs = {k: (None if coeffs.get(k) is None else np.asarray(coeffs[k]))
                            for k in O.Problem2D.OPS}
        src = np.asarray(source)
        self.multi = src.ndim == 3
        self.source = src if self.multi else src[..., None]
        self.L = L
        self.run = Runner(threads)

    @property
    def boundary_points(self):
        return self.base.boundary_points

    @property
    def points(self):
        return self.base.points

    def build(self):
        b = self.base
        self.Y, T, self.v, h = leaf_stage_dtn(b.coeffs, b.ops, self.source, b.P, b.Q, self.run)
        self.S_lst, self.g_lst, self.T_top, self.h_top = merge_stage_dtn(T, h, self.L, self.run)
        return self

    def solve(self, bdry):
        bd = np.asarray(bdry, dtype=np.float64)
        b2 = bd if bd.ndim == 2 else bd[:, None]
        u = down_pass_dtn(b2, self.S_lst, self.g_lst, self.Y, self.v, self.run)
        return u if self.multi else u[..., 0]

    def close(self):
        self.run.close()

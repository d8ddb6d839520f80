"""Loading and comparing the golden fixtures under ``tests/golden/``.

The fixtures are outputs of the unmodified reference package (meliao/jaxhps)
written by ``tests/golden/make_fixtures.py``.  Matrices larger than 1 MB are
stored as ``M @ probe`` (``<key>_probe``) plus every 16th row
(``<key>_rows16``), with the probe rebuilt here from the same seed.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
PROBE_SEED = 99


def load(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def probe_matrix(n_cols: int, n_probe: int = 4) -> np.ndarray:
    return np.random.default_rng(PROBE_SEED).standard_normal((n_cols, n_probe))


def to_np(a) -> np.ndarray:
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    return np.asarray(a)


def same_points(a, b) -> bool:
    """Grid points agree to a few units in the last place (the Gauss nodes
    come from an eigenvalue solver whose last bits differ between CPU
    architectures)."""
    a, b = to_np(a), to_np(b)
    return a.shape == b.shape and float(np.abs(a - b).max()) <= 1e-15 * max(1.0, float(np.abs(b).max()))


def rel(a, b) -> float:
    """max |a - b| / max |b|."""
    a, b = to_np(a), to_np(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def rel_l2(a, b) -> float:
    a, b = to_np(a), to_np(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def matrix_err(fx: dict, key: str, M) -> float:
    """Relative error of M against the fixture's ``key`` (dense, or probe +
    row sample for large matrices)."""
    M = to_np(M)
    if key in fx:
        return rel(M.reshape(fx[key].shape), fx[key])
    P = probe_matrix(M.shape[-1])
    e1 = rel(M @ P, fx[key + "_probe"].reshape((M @ P).shape))
    e2 = rel(M[..., ::16, :], fx[key + "_rows16"].reshape(M[..., ::16, :].shape))
    return max(e1, e2)

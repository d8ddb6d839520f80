"""Interpolation between the HPS grid and rectangular grids (API mirror of
src/jaxhps/_interpolation_methods.py:23-340 and Domain.interp_* in
src/jaxhps/_domain.py:99-294).

The arithmetic runs in the native library (``hps_interp_rows``,
``hps_gather_cols``, ``hps_interp_from_leaves`` and batched GEMMs); host code
builds the small per-leaf node arrays, the barycentric weights and a table
of the finest cells of the root box for locating target points.

Conventions kept from the reference:
* 2D leaf grids have y descending (the leaf's x nodes ascending, y nodes
  flipped); 3D grids are ascending on every axis.
* ``interp_from_hps_2D`` builds its targets with ``meshgrid(x, y)`` (default
  'xy' indexing, shape (n_y, n_x)) and returns the values reshaped to
  (n_x, n_y); ``interp_from_hps_3D`` likewise with (n_y, n_x, n_z) targets
  and (n_x, n_y, n_z) values.
* A target outside every leaf takes leaf 0.
"""

from __future__ import annotations

import ctypes as C
from typing import Sequence, Tuple

import numpy as np
import torch

from . import _native as nat
from . import _stages as st
from ._quadrature import chebyshev_points


def _bary_weights(x: np.ndarray) -> np.ndarray:
    diff = x[:, None] - x[None, :]
    np.fill_diagonal(diff, 1.0)
    return np.prod(diff, axis=0)


def _rearrange(p: int, dim: int) -> np.ndarray:
    if dim == 2:
        from ._grid_creation_2D import rearrange_indices_ext_int
    else:
        from ._grid_creation_3D import rearrange_indices_ext_int
    return np.asarray(rearrange_indices_ext_int(p), dtype=np.int32)


def _leaf_bounds(leaves) -> np.ndarray:
    if isinstance(leaves, np.ndarray):
        return np.asarray(leaves, dtype=np.float64)
    if isinstance(leaves, torch.Tensor):
        return leaves.detach().cpu().numpy().astype(np.float64)
    rows = []
    for n in leaves:
        if hasattr(n, "zmin"):
            rows.append([n.xmin, n.xmax, n.ymin, n.ymax, n.zmin, n.zmax])
        else:
            rows.append([n.xmin, n.xmax, n.ymin, n.ymax])
    return np.asarray(rows, dtype=np.float64)


def _leaf_nodes(bounds: np.ndarray, p: int, dim: int) -> Tuple[np.ndarray, np.ndarray]:
    """(n_leaves, dim, p) interpolation nodes per axis and their weights."""
    c = chebyshev_points(p)
    nl = bounds.shape[0]
    nodes = np.empty((nl, dim, p))
    for a in range(dim):
        lo, hi = bounds[:, 2 * a:2 * a + 1], bounds[:, 2 * a + 1:2 * a + 2]
        nodes[:, a, :] = 0.5 * (hi - lo) * c[None, :] + 0.5 * (lo + hi)   # affine_transform, per leaf
    if dim == 2:
        nodes[:, 1, :] = nodes[:, 1, ::-1]
    diff = nodes[:, :, :, None] - nodes[:, :, None, :]
    idx = np.arange(p)
    diff[:, :, idx, idx] = 1.0
    wts = np.prod(diff, axis=2)
    return np.ascontiguousarray(nodes), np.ascontiguousarray(wts)


def _cell_table(bounds: np.ndarray, dim: int, max_cells: int = 1 << 26):
    """Leaf index of every finest cell of the root box.  Returns (cells (int32,
    C-order over the axes), n_cells, origin, cell sizes)."""
    lo = np.array([bounds[:, 2 * a].min() for a in range(dim)])
    hi = np.array([bounds[:, 2 * a + 1].max() for a in range(dim)])
    h = np.array([(bounds[:, 2 * a + 1] - bounds[:, 2 * a]).min() for a in range(dim)])
    nc = np.maximum(1, np.rint((hi - lo) / h).astype(np.int64))
    if int(np.prod(nc)) > max_cells:
        raise NotImplementedError("interpolation: the tree is too deep for the cell table")
    h = (hi - lo) / nc
    cells = np.full(tuple(int(n) for n in nc), -1, dtype=np.int32)
    for leaf, b in enumerate(bounds):
        sl = []
        for a in range(dim):
            i0 = int(np.rint((b[2 * a] - lo[a]) / h[a]))
            i1 = int(np.rint((b[2 * a + 1] - lo[a]) / h[a]))
            sl.append(slice(max(i0, 0), max(min(i1, int(nc[a])), i0 + 1)))
        cells[tuple(sl)] = leaf
    if (cells < 0).any():
        raise ValueError("interpolation: the leaves do not tile their bounding box")
    return np.ascontiguousarray(cells), nc.astype(np.int32), lo, h


def _device_f64(x, dev) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.to(device=dev, dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(np.asarray(x, dtype=np.float64)), device=dev)


def _from_hps(bounds: np.ndarray, p: int, f_evals, targets: np.ndarray, dim: int, device=None) -> torch.Tensor:
    L = nat.lib()
    dev = st._device(device)
    f = f_evals if isinstance(f_evals, torch.Tensor) else torch.as_tensor(np.asarray(f_evals))
    if f.is_complex():
        re = _from_hps(bounds, p, f.real, targets, dim, device)
        im = _from_hps(bounds, p, f.imag, targets, dim, device)
        return torch.complex(re, im)
    f = _device_f64(f, dev)
    nl = bounds.shape[0]
    if f.shape[0] != nl or f.shape[1] != p ** dim:
        raise ValueError(f"f_evals has shape {tuple(f.shape)}, expected ({nl}, {p ** dim}[, n_src])")
    ns = f.shape[2] if f.dim() == 3 else 1
    nodes, wts = _leaf_nodes(bounds, p, dim)
    cells, nc, lo, h = _cell_table(bounds, dim)
    tb, tn, tw = (_device_f64(x, dev) for x in (bounds, nodes, wts))
    tr = torch.as_tensor(_rearrange(p, dim), device=dev)
    tc = torch.as_tensor(cells, device=dev)
    tt = _device_f64(targets.reshape(-1, dim), dev)
    out = torch.empty((tt.shape[0], ns), dtype=torch.float64, device=dev)
    ncb = (C.c_int * dim)(*[int(x) for x in nc])
    lob = (C.c_double * dim)(*[float(x) for x in lo])
    hb = (C.c_double * dim)(*[float(x) for x in h])
    nat.check(L.hps_interp_from_leaves(dim, tt.shape[0], ns, tt.data_ptr(), p, tb.data_ptr(), tn.data_ptr(),
                                       tw.data_ptr(), tr.data_ptr(), tc.data_ptr(), ncb, lob, hb, f.data_ptr(),
                                       out.data_ptr(), nat.stream_ptr()), "hps_interp_from_leaves")
    return out if f.dim() == 3 else out[:, 0]


def interp_from_hps_2D(leaves, p: int, f_evals, x_vals, y_vals, device=None, host_device="cpu"):
    """Values of the HPS function f_evals (n_leaves, p^2[, n_src]) on
    meshgrid(x_vals, y_vals); returns (vals (n_x, n_y[, n_src]),
    target_pts (n_y, n_x, 2)) (reference _interpolation_methods.py:23-94)."""
    x = np.asarray(x_vals.cpu() if isinstance(x_vals, torch.Tensor) else x_vals, dtype=np.float64)
    y = np.asarray(y_vals.cpu() if isinstance(y_vals, torch.Tensor) else y_vals, dtype=np.float64)
    X, Y = np.meshgrid(x, y)
    target = np.stack([X, Y], axis=2)
    vals = _from_hps(_leaf_bounds(leaves), p, f_evals, target, 2, device)
    shape = (x.shape[0], y.shape[0]) + tuple(vals.shape[1:])
    return st._to_host(vals.reshape(shape), host_device), target


def interp_from_hps_3D(leaves, p: int, f_evals, x_vals, y_vals, z_vals, device=None, host_device="cpu"):
    """3D analogue (reference :144-225): targets meshgrid(x, y, z) with
    shape (n_y, n_x, n_z, 3), values reshaped to (n_x, n_y, n_z[, n_src])."""
    x, y, z = (np.asarray(v.cpu() if isinstance(v, torch.Tensor) else v, dtype=np.float64)
               for v in (x_vals, y_vals, z_vals))
    X, Y, Z = np.meshgrid(x, y, z)
    target = np.stack([X, Y, Z], axis=3)
    vals = _from_hps(_leaf_bounds(leaves), p, f_evals, target, 3, device)
    shape = (x.shape[0], y.shape[0], z.shape[0]) + tuple(vals.shape[1:])
    return st._to_host(vals.reshape(shape), host_device), target


def _rows(to_pts: np.ndarray, src: np.ndarray, p: int, transposed: bool, dev) -> torch.Tensor:
    """1D interpolation rows from src to every leaf's p nodes (to_pts
    (n_leaves, p)): (n_leaves * p, n_src), or (n_leaves, n_src, p) when
    transposed."""
    L = nat.lib()
    nl = to_pts.shape[0]
    tt = _device_f64(to_pts.reshape(-1), dev)
    ts = _device_f64(src, dev)
    tw = _device_f64(_bary_weights(src), dev)
    out = torch.empty((nl, src.shape[0], p) if transposed else (nl * p, src.shape[0]), dtype=torch.float64,
                      device=dev)
    nat.check(L.hps_interp_rows(nl * p, src.shape[0], tt.data_ptr(), ts.data_ptr(), tw.data_ptr(), out.data_ptr(), p,
                                int(transposed), nat.stream_ptr()), "hps_interp_rows")
    return out


def _to_hps(bounds: np.ndarray, samples, p: int, axes: Sequence[np.ndarray], device=None) -> torch.Tensor:
    L = nat.lib()
    dev = st._device(device)
    dim = len(axes)
    V = samples if isinstance(samples, torch.Tensor) else torch.as_tensor(np.asarray(samples))
    if V.is_complex():
        return torch.complex(_to_hps(bounds, V.real, p, axes, device), _to_hps(bounds, V.imag, p, axes, device))
    V = _device_f64(V, dev)
    n = [a.shape[0] for a in axes]
    if tuple(V.shape) != tuple(n):
        raise ValueError(f"values have shape {tuple(V.shape)}, expected {tuple(n)}")
    nl = bounds.shape[0]
    c = chebyshev_points(p)
    to = [0.5 * (bounds[:, 2 * a + 1:2 * a + 2] - bounds[:, 2 * a:2 * a + 1]) * c[None, :]
          + 0.5 * (bounds[:, 2 * a:2 * a + 1] + bounds[:, 2 * a + 1:2 * a + 2]) for a in range(dim)]
    if dim == 2:
        to[1] = np.ascontiguousarray(to[1][:, ::-1])
    Mx = _rows(to[0], axes[0], p, False, dev)                        # (nl p, n_x)
    ppd = p ** dim
    O = torch.empty((nl, ppd), dtype=torch.float64, device=dev)
    if dim == 2:
        T = torch.empty((nl * p, n[1]), dtype=torch.float64, device=dev)
        nat.gemm(Mx, V, T)                                             # contract x
        MyT = _rows(to[1], axes[1], p, True, dev)                     # (nl, n_y, p)
        nat.gemm(T.view(nl, p, n[1]), MyT, O.view(nl, p, p))          # contract y
    else:
        T1 = torch.empty((nl * p, n[1] * n[2]), dtype=torch.float64, device=dev)
        nat.gemm(Mx, V.reshape(n[0], n[1] * n[2]), T1)                 # contract x
        My = _rows(to[1], axes[1], p, False, dev).view(nl, p, n[1])
        MzT = _rows(to[2], axes[2], p, True, dev)                     # (nl, n_z, p)
        T1v = T1.view(nl, p, n[1], n[2])
        T2 = torch.empty((nl, p, n[2]), dtype=torch.float64, device=dev)
        Ov = O.view(nl, p, p, p)
        for ix in range(p):
            nat.gemm(My, T1v[:, ix], T2)                               # contract y
            nat.gemm(T2, MzT, Ov[:, ix])                               # contract z
    out = torch.empty((nl, ppd), dtype=torch.float64, device=dev)
    tr = torch.as_tensor(_rearrange(p, dim), device=dev)
    nat.check(L.hps_gather_cols(nl, ppd, ppd, tr.data_ptr(), O.data_ptr(), out.data_ptr(), nat.stream_ptr()),
              "hps_gather_cols")
    return out


def interp_to_hps_2D(leaf_bounds, samples, p: int, from_x, from_y, device=None, host_device="cpu"):
    """Values on every leaf's grid (n_leaves, p^2) of the interpolant of
    samples (n_x, n_y) given on meshgrid(from_x, from_y, indexing='ij')
    (reference interp_to_single_Chebyshev_panel_2D, :228-263, vmapped)."""
    ax = [np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a, dtype=np.float64) for a in (from_x, from_y)]
    return st._to_host(_to_hps(_leaf_bounds(leaf_bounds), samples, p, ax, device), host_device)


def interp_to_hps_3D(leaf_bounds, samples, p: int, from_x, from_y, from_z, device=None, host_device="cpu"):
    """3D analogue (reference :271-302): samples (n_x, n_y, n_z)."""
    ax = [np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a, dtype=np.float64) for a in (from_x, from_y, from_z)]
    return st._to_host(_to_hps(_leaf_bounds(leaf_bounds), samples, p, ax, device), host_device)

"""ctypes binding of the native library (C ABI: include/jaxhps_gb300.h).

The product path has no CPU fallback: if ``libjaxhps_gb300.so`` is missing
or CUDA is unavailable, every stage raises.  Device memory comes from torch
tensors; their ``data_ptr()`` values are passed straight to the C ABI along
with torch's current CUDA stream.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import torch

_LIB_PATH = Path(__file__).resolve().parent / "libjaxhps_gb300.so"
_lock = threading.Lock()
_lib = None

HPS_F64, HPS_F32, HPS_C128, HPS_C64 = 0, 1, 2, 3
HPS_CODE_PAD = -(2 ** 31)
HPS_UP_B_IS_BD_INV, HPS_UP_ITI = 1, 2

TORCH_TO_HPS = {
    torch.float64: HPS_F64,
    torch.float32: HPS_F32,
    torch.complex128: HPS_C128,
    torch.complex64: HPS_C64,
}


class NativeError(RuntimeError):
    """A native-library call returned a non-zero status."""


class SingularPivotError(NativeError):
    """A batched inverse met an exactly zero pivot (info > 0): the matrix is
    singular and the operators built from it are not finite."""


class DeviceWaitTimeout(NativeError):
    """A bounded device wait ran out (info = -1 from a multi-CTA inverse
    panel, or the tensor-core GEMM's flag); the results are invalid."""


class RefinementNotConverged(NativeError):
    """Iterative refinement used its step budget without reaching the
    requested tolerance."""


vp = C.c_void_p
ci = C.c_int
cll = C.c_longlong
csz = C.c_size_t


class LeafDtnArgs(C.Structure):
    _fields_ = [
        ("dtype", ci), ("coef_complex", ci), ("n_leaves", ci), ("n_pts", ci), ("n_cb", ci),
        ("n_gauss", ci), ("nsrc", ci), ("n_ops", ci),
        ("ops", vp), ("coeffs", vp), ("source", vp), ("P", vp), ("Q", vp),
        ("Y", vp), ("T", vp), ("v", vp), ("h", vp), ("Aii_inv", vp), ("info", vp),
        ("workspace", vp), ("workspace_bytes", csz),
    ]


class LeafItiArgs(C.Structure):
    _fields_ = [
        ("dtype", ci), ("coef_complex", ci), ("n_leaves", ci), ("n_pts", ci), ("n_cb", ci),
        ("n_gauss", ci), ("nsrc", ci), ("n_ops", ci),
        ("ops", vp), ("coeffs", vp), ("source", vp), ("G", vp), ("P", vp), ("QH", vp),
        ("Y", vp), ("T", vp), ("v", vp), ("h", vp), ("B_inv", vp), ("info", vp),
        ("workspace", vp), ("workspace_bytes", csz),
    ]


class MergeArgs(C.Structure):
    _fields_ = [
        ("dtype", ci), ("n_merges", ci), ("nch", ci), ("nb", ci), ("n_int", ci), ("n_ext", ci),
        ("nsrc", ci),
        ("T_children", vp), ("h_children", vp),
        ("int_c", vp), ("int_l", vp), ("ext_c", vp), ("ext_l", vp), ("loc", vp),
        ("S", vp), ("g_tilde", vp), ("T_out", vp), ("h_out", vp), ("D_inv", vp), ("BD_inv", vp),
        ("B_out", vp), ("info", vp), ("workspace", vp), ("workspace_bytes", csz),
        ("n_c_rects", ci), ("c_rects", vp), ("n_b_rects", ci), ("b_rects", vp),
        ("n_x", ci), ("colour_perm", vp),
    ]


class UpArgs(C.Structure):
    _fields_ = [
        ("dtype", ci), ("n_merges", ci), ("nch", ci), ("nb", ci), ("n_int", ci), ("n_ext", ci), ("nsrc", ci),
        ("h_children", vp), ("int_c", vp), ("int_l", vp), ("ext_c", vp), ("ext_l", vp),
        ("D_inv", vp), ("B", vp), ("dh", vp), ("g_tilde", vp), ("h_out", vp), ("flags", ci),
    ]


class Residual2DArgs(C.Structure):
    _fields_ = [
        ("n_leaves", ci), ("p", ci), ("q", ci), ("nsrc", ci), ("n_ops", ci), ("op_kind", ci * 10),
        ("coeffs", vp), ("inv_half", vp), ("D1", vp), ("D2", vp), ("Pside", vp), ("Qside", vp), ("perm", vp),
        ("u_int", vp), ("g", vp), ("f", vp), ("r_int", vp), ("r_int64", vp), ("flux", vp), ("u_full", vp),
    ]


class ResidualIti2DArgs(C.Structure):
    _fields_ = [
        ("n_leaves", ci), ("p", ci), ("q", ci), ("nsrc", ci), ("n_ops", ci), ("op_kind", ci * 10),
        ("coef_complex", ci), ("eta", C.c_double),
        ("coeffs", vp), ("inv_half", vp), ("D1", vp), ("D2", vp), ("Pside", vp), ("Qside", vp), ("perm", vp),
        ("u", vp), ("t_in", vp), ("f", vp), ("r", vp), ("t_out", vp),
    ]


class DownArgs(C.Structure):
    _fields_ = [
        ("dtype", ci), ("n_merges", ci), ("nch", ci), ("nb", ci), ("n_int", ci), ("n_ext", ci),
        ("nsrc", ci),
        ("S", vp), ("g_tilde", vp), ("g_parent", vp), ("code", vp), ("g_int", vp), ("g_children", vp),
    ]


def _declare(lib):
    P = C.POINTER
    lib.hps_version.restype = C.c_char_p
    lib.hps_launch_count.restype = cll
    lib.hps_profile_begin.argtypes = [ci]
    lib.hps_profile_begin.restype = ci
    lib.hps_profile_end.argtypes = [P(C.c_double), P(cll), P(C.c_double)]
    lib.hps_profile_end.restype = ci
    lib.hps_last_error.argtypes = [C.c_char_p, csz]
    lib.hps_last_error.restype = ci
    lib.hps_gemm_batched.argtypes = [ci, ci, ci, ci, P(C.c_double), vp, cll, cll, vp, cll, cll, P(C.c_double),
                                     vp, cll, cll, vp, cll, cll, ci, vp]
    lib.hps_gemm_batched.restype = ci
    lib.hps_inverse_workspace_size.argtypes = [ci, ci, ci]
    lib.hps_inverse_workspace_size.restype = csz
    lib.hps_inverse_batched.argtypes = [ci, ci, vp, cll, cll, vp, cll, cll, ci, vp, vp, csz, vp]
    lib.hps_inverse_batched.restype = ci
    lib.hps_convert.argtypes = [ci, ci, cll, vp, vp, vp]
    lib.hps_convert.restype = ci
    lib.hps_local_solve_dtn_workspace_size.argtypes = [P(LeafDtnArgs)]
    lib.hps_local_solve_dtn_workspace_size.restype = csz
    lib.hps_local_solve_dtn.argtypes = [P(LeafDtnArgs), vp]
    lib.hps_local_solve_dtn.restype = ci
    lib.hps_local_solve_iti_workspace_size.argtypes = [P(LeafItiArgs)]
    lib.hps_local_solve_iti_workspace_size.restype = csz
    lib.hps_local_solve_iti.argtypes = [P(LeafItiArgs), vp]
    lib.hps_local_solve_iti.restype = ci
    lib.hps_merge_level_dtn_workspace_size.argtypes = [P(MergeArgs)]
    lib.hps_merge_level_dtn_workspace_size.restype = csz
    lib.hps_merge_level_dtn.argtypes = [P(MergeArgs), vp]
    lib.hps_merge_level_dtn.restype = ci
    lib.hps_merge_level_iti.argtypes = [P(MergeArgs), vp]
    lib.hps_merge_level_iti.restype = ci
    lib.hps_down_level.argtypes = [P(DownArgs), vp]
    lib.hps_down_level.restype = ci
    lib.hps_up_level.argtypes = [P(UpArgs), vp]
    lib.hps_up_level.restype = ci
    lib.hps_residual_2d.argtypes = [P(Residual2DArgs), vp]
    lib.hps_residual_2d.restype = ci
    lib.hps_flux_combine.argtypes = [cll, ci, vp, vp, vp, ci, vp, vp, vp, vp, vp]
    lib.hps_flux_combine.restype = ci
    lib.hps_accumulate.argtypes = [cll, vp, vp, vp]
    lib.hps_accumulate.restype = ci
    lib.hps_residual_update_2d.argtypes = [P(Residual2DArgs), vp, vp, vp]
    lib.hps_residual_update_2d.restype = ci
    lib.hps_residual_2d_df.argtypes = [P(Residual2DArgs), vp, vp, vp]
    lib.hps_accumulate_max_df.argtypes = [cll, vp, vp, vp, vp, vp]
    lib.hps_accumulate_max_df.restype = ci
    lib.hps_assemble_u_2d_df.argtypes = [ci, ci, ci, ci, vp, vp, vp, vp, vp, vp]
    lib.hps_assemble_u_2d_df.restype = ci
    lib.hps_residual_2d_df.restype = ci
    lib.hps_residual_update_2d_df.argtypes = [P(Residual2DArgs), vp, vp, vp, vp, vp]
    lib.hps_residual_update_2d_df.restype = ci
    lib.hps_residual_df_prep_size.argtypes = [ci, ci, ci, ci]
    lib.hps_residual_df_prep_size.restype = csz
    lib.hps_residual_df_prepare.argtypes = [P(Residual2DArgs), vp, vp]
    lib.hps_residual_df_prepare.restype = ci
    lib.hps_inverse_interface.argtypes = lib.hps_inverse_batched.argtypes
    lib.hps_inverse_interface.restype = ci
    lib.hps_mapped_pointer.argtypes = [vp, P(vp)]
    lib.hps_mapped_pointer.restype = ci
    lib.hps_inverse_block_policy.argtypes = [ci]
    lib.hps_inverse_block_policy.restype = ci
    lib.hps_residual_df_supported.argtypes = [ci, ci]
    lib.hps_residual_df_supported.restype = ci
    lib.hps_assemble_u_2d.argtypes = [ci, ci, ci, ci, vp, vp, vp, vp, vp]
    lib.hps_assemble_u_2d.restype = ci
    lib.hps_interior_f32.argtypes = [cll, ci, ci, ci, vp, vp, vp]
    lib.hps_interior_f32.restype = ci
    lib.hps_assemble_rows.argtypes = [ci, ci, ci, ci, ci, vp, vp, vp, cll, cll, vp]
    lib.hps_assemble_rows.restype = ci
    lib.hps_refine_points_3d.argtypes = [ci, ci, vp, vp, vp, vp, vp]
    lib.hps_refine_points_3d.restype = ci
    lib.hps_refine_points_2d.argtypes = [ci, ci, vp, vp, vp, vp, vp]
    lib.hps_refine_points_2d.restype = ci
    lib.hps_refine_check_3d.argtypes = [ci, ci, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    lib.hps_refine_check_3d.restype = ci
    lib.hps_refine_check_2d.argtypes = [ci, ci, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    lib.hps_refine_check_2d.restype = ci
    lib.hps_panel_map.argtypes = [ci, ci, ci, ci, ci, ci, vp, vp, vp, cll, cll, vp, cll, cll, vp]
    lib.hps_panel_map.restype = ci
    lib.hps_scale_batched.argtypes = [ci, ci, cll, vp, vp, vp]
    lib.hps_scale_batched.restype = ci
    lib.hps_iti_combine.argtypes = [cll, ci, vp, vp, vp, vp, ci, vp, vp, vp, vp]
    lib.hps_iti_combine.restype = ci
    lib.hps_residual_iti_2d.argtypes = [P(ResidualIti2DArgs), vp]
    lib.hps_residual_iti_2d.restype = ci
    lib.hps_accumulate_max.argtypes = [cll, ci, vp, vp, vp, vp]
    lib.hps_accumulate_max.restype = ci
    lib.hps_gemm_policy.argtypes = [ci]
    lib.hps_gemm_policy.restype = ci
    lib.hps_interp_rows.argtypes = [cll, ci, vp, vp, vp, vp, ci, ci, vp]
    lib.hps_interp_rows.restype = ci
    lib.hps_gather_cols.argtypes = [cll, ci, ci, vp, vp, vp, vp]
    lib.hps_gather_cols.restype = ci
    lib.hps_interp_from_leaves.argtypes = [ci, cll, ci, vp, ci, vp, vp, vp, vp, vp, P(ci), P(C.c_double),
                                           P(C.c_double), vp, vp, vp]
    lib.hps_interp_from_leaves.restype = ci
    lib.hps_assemble_rows_complex.argtypes = [ci, ci, ci, ci, ci, vp, vp, vp, cll, cll, vp]
    lib.hps_assemble_rows_complex.restype = ci
    lib.hps_gemm_tc_status.argtypes = []
    lib.hps_gemm_tc_status.restype = ci
    lib.hps_gemm_tc_status_reset.argtypes = []
    lib.hps_gemm_tc_status_reset.restype = ci
    lib.hps_gemm_tune_set.argtypes = [ci, ci, ci, ci, ci]
    lib.hps_gemm_tune_set.restype = ci
    lib.hps_gemm_tune_clear.argtypes = []
    lib.hps_gemm_tune_clear.restype = ci
    lib.hps_gemm_force_variant.argtypes = [ci]
    lib.hps_gemm_force_variant.restype = ci
    lib.hps_gemm_shapes.argtypes = [ci, P(cll), cll]
    lib.hps_gemm_shapes.restype = cll
    lib.hps_inverse_policy.argtypes = [ci]
    lib.hps_inverse_policy.restype = ci
    lib.hps_set_spin_limits.argtypes = [cll, cll, P(cll), P(cll)]
    lib.hps_set_spin_limits.restype = ci
    lib.hps_mlp_param_count.argtypes = []
    lib.hps_mlp_param_count.restype = ci
    lib.hps_mlp_sample_points.argtypes = [ci, vp, vp, vp]
    lib.hps_mlp_sample_points.restype = ci
    lib.hps_mlp_features.argtypes = [ci, vp, vp, C.c_double, vp, vp]
    lib.hps_mlp_features.restype = ci
    lib.hps_mlp_forward.argtypes = [ci, vp, vp, vp, vp, vp, vp]
    lib.hps_mlp_forward.restype = ci
    lib.hps_mlp_bce.argtypes = [ci, vp, vp, C.c_float, vp, vp, vp]
    lib.hps_mlp_bce.restype = ci
    lib.hps_mlp_backward.argtypes = [ci, vp, vp, vp, vp, vp, vp, vp]
    lib.hps_mlp_backward.restype = ci
    lib.hps_mlp_adam.argtypes = [vp, vp, vp, vp, C.c_float, C.c_float, C.c_float, C.c_float, ci, vp]
    lib.hps_mlp_adam.restype = ci


EXPORTED_SYMBOLS = (
    "hps_version", "hps_launch_count", "hps_profile_begin", "hps_profile_end", "hps_last_error", "hps_gemm_batched", "hps_inverse_workspace_size",
    "hps_inverse_batched", "hps_convert", "hps_local_solve_dtn_workspace_size", "hps_local_solve_dtn",
    "hps_local_solve_iti_workspace_size", "hps_local_solve_iti", "hps_merge_level_dtn_workspace_size",
    "hps_merge_level_dtn", "hps_merge_level_iti", "hps_down_level", "hps_up_level", "hps_residual_2d", "hps_flux_combine",
    "hps_accumulate", "hps_residual_update_2d", "hps_residual_2d_df", "hps_residual_update_2d_df",
    "hps_residual_df_supported", "hps_residual_df_prep_size", "hps_inverse_block_policy", "hps_inverse_interface", "hps_mapped_pointer", "hps_accumulate_max_df",
    "hps_assemble_u_2d_df", "hps_residual_df_prepare", "hps_assemble_u_2d", "hps_interior_f32", "hps_assemble_rows",
    "hps_refine_points_3d", "hps_refine_check_3d", "hps_mlp_param_count", "hps_mlp_sample_points",
    "hps_mlp_features", "hps_mlp_forward", "hps_mlp_bce", "hps_mlp_backward", "hps_mlp_adam", "hps_panel_map",
    "hps_scale_batched", "hps_gemm_tc_status", "hps_gemm_tc_status_reset", "hps_set_spin_limits", "hps_inverse_policy", "hps_gemm_tune_set", "hps_gemm_tune_clear", "hps_gemm_force_variant", "hps_gemm_shapes", "hps_iti_combine", "hps_residual_iti_2d", "hps_gemm_policy", "hps_accumulate_max", "hps_refine_points_2d", "hps_refine_check_2d", "hps_interp_rows", "hps_gather_cols", "hps_interp_from_leaves", "hps_assemble_rows_complex",
)


def load_library(path: Path | None = None):
    """Loads (without building) the shared library; raises if it is absent."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path is not None else _LIB_PATH
        if not p.exists():
            raise NativeError(
                f"native library {p} not found: build it with `python -c \"import __graft_entry__ as g; g.build()\"`"
            )
        lib = C.CDLL(str(p))
        _declare(lib)
        if path is None:
            _lib = lib
        return lib


def lib():
    """The loaded library, for GPU work.  Raises if CUDA is unavailable."""
    if not torch.cuda.is_available():
        raise NativeError("jaxhps_gb300 needs a CUDA device; no CPU fallback exists")
    return load_library()


def check(status: int, what: str) -> None:
    if status != 0:
        buf = C.create_string_buffer(1024)
        load_library().hps_last_error(buf, 1024)
        raise NativeError(f"{what} failed with status {status}: {buf.value.decode(errors='replace')}")


def set_spin_limits(panel_barrier_polls: int = -1, tc_wait_polls: int = -1):
    """Sets the bounded waits' poll limits on the current device (negative:
    keep); returns the previous (panel_barrier_polls, tc_wait_polls)."""
    a, b = C.c_longlong(0), C.c_longlong(0)
    check(lib().hps_set_spin_limits(int(panel_barrier_polls), int(tc_wait_polls), C.byref(a), C.byref(b)),
          "hps_set_spin_limits")
    return int(a.value), int(b.value)


def raise_on_tc_timeout(what: str) -> None:
    """Reads and clears the tensor-core GEMM's timeout flag (one device sync);
    raises DeviceWaitTimeout when a wait ran out since the last check."""
    torch.cuda.current_stream().synchronize()
    if lib().hps_gemm_tc_status_reset() != 0:
        raise DeviceWaitTimeout(f"{what}: a tensor-core GEMM's bounded wait ran out; the results are invalid")


def launch_count() -> int:
    """Kernels enqueued by the native library so far (process-wide)."""
    return int(load_library().hps_launch_count())


KC_GEMM, KC_INVERSE, KC_MOVE, KC_RESIDUAL, KC_GEMM_TMA, KC_RESIDUAL_DF, KC_INVERSE_TC = 1, 2, 3, 4, 5, 6, 7


def profile_begin(*kernel_classes: int) -> None:
    mask = 0
    for c in kernel_classes:
        mask |= 1 << c
    check(load_library().hps_profile_begin(mask), "hps_profile_begin")


def profile_end():
    """{class: (summed kernel ms, launches, summed algorithmic work)} since profile_begin."""
    ms, n, w = (C.c_double * 8)(), (C.c_longlong * 8)(), (C.c_double * 8)()
    check(load_library().hps_profile_end(ms, n, w), "hps_profile_end")
    return {c: (ms[c], n[c], w[c]) for c in range(1, 8) if n[c]}


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


class Workspace:
    """Grow-only device scratch buffer reused across calls."""

    def __init__(self):
        self.buf = None

    def get(self, nbytes: int, device) -> torch.Tensor:
        nbytes = max(int(nbytes), 256)
        if self.buf is None or self.buf.numel() < nbytes or self.buf.device != torch.device(device):
            self.buf = None
            self.buf = torch.empty(nbytes, dtype=torch.uint8, device=device)
        return self.buf


_ws = Workspace()


def workspace(nbytes: int, device) -> torch.Tensor:
    return _ws.get(nbytes, device)


def release_workspace() -> None:
    _ws.buf = None


# ---------------------------------------------------------------------------
# thin wrappers over the primitives
# ---------------------------------------------------------------------------


def gemm(A, B, out, alpha=1.0, beta=0.0, Cmat=None, batch=None):
    """out[b] = alpha A[b] @ B[b] + beta C[b] for 3D (or broadcast 2D) tensors,
    all contiguous in their last two dims."""
    L = lib()
    dt = TORCH_TO_HPS[out.dtype]

    def mat(t):
        if t.dim() == 2:
            return t.shape[0], t.shape[1], t.stride(0), 0
        return t.shape[1], t.shape[2], t.stride(1), t.stride(0)

    m, k, lda, sA = mat(A)
    k2, n, ldb, sB = mat(B)
    assert k == k2, (A.shape, B.shape)
    mo, no, ldd, sD = mat(out)
    assert (mo, no) == (m, n)
    nb = batch if batch is not None else (out.shape[0] if out.dim() == 3 else 1)
    al = (C.c_double * 2)(complex(alpha).real, complex(alpha).imag)
    be = (C.c_double * 2)(complex(beta).real, complex(beta).imag)
    if Cmat is not None:
        _, _, ldc, sC = mat(Cmat)
        cp = Cmat.data_ptr()
    else:
        ldc, sC, cp = 0, 0, None
    check(L.hps_gemm_batched(dt, m, n, k, al, A.data_ptr(), lda, sA, B.data_ptr(), ldb, sB, be, cp, ldc, sC,
                             out.data_ptr(), ldd, sD, nb, stream_ptr()), "hps_gemm_batched")
    return out


def accumulate_max_df(x: torch.Tensor, y_hi: torch.Tensor, y_lo: torch.Tensor, out: torch.Tensor):
    """(y_hi, y_lo) += x in double-float and (max |x|, max |y|) as two Python
    floats (one device sync)."""
    check(lib().hps_accumulate_max_df(x.numel(), x.data_ptr(), y_hi.data_ptr(), y_lo.data_ptr(), out.data_ptr(),
                                      stream_ptr()), "hps_accumulate_max_df")
    mx, my = out.tolist()
    return mx, my


def mapped_pointer(t: torch.Tensor):
    """Device address of a page-locked CPU tensor's memory, or None when the
    tensor is not page-locked (mapped) memory."""
    if t.device.type != "cpu" or not t.is_pinned():
        return None
    dp = C.c_void_p()
    if lib().hps_mapped_pointer(t.data_ptr(), C.byref(dp)) != 0:
        return None
    return dp.value


def inverse(A, out=None, info=None, entry="hps_inverse_batched"):
    """Batched inverse of a (batch, n, n) tensor (out may be A); entry
    "hps_inverse_interface" selects the merge interface-matrix inverse."""
    L = lib()
    if A.dim() == 2:
        A = A.unsqueeze(0)
    if out is None:
        out = torch.empty_like(A)
    b, n, _ = A.shape
    dt = TORCH_TO_HPS[A.dtype]
    wsb = L.hps_inverse_workspace_size(dt, n, b)
    ws = workspace(wsb, A.device) if wsb else None
    check(getattr(L, entry)(dt, n, A.data_ptr(), A.stride(1), A.stride(0), out.data_ptr(), out.stride(1),
                            out.stride(0), b, ptr(info), ptr(ws), wsb, stream_ptr()), entry)
    return out


def accumulate_max(x: torch.Tensor, y: torch.Tensor, out: torch.Tensor, pairs: bool = False):
    """y += x (FP32 into FP64, or complex64 into complex128 with pairs) and
    (max |x|, max |y|) as two Python floats (one device sync)."""
    xf = torch.view_as_real(x) if x.is_complex() else x
    check(lib().hps_accumulate_max(xf.numel(), int(pairs), x.data_ptr(), y.data_ptr(), out.data_ptr(), stream_ptr()),
          "hps_accumulate_max")
    mx, my = out.tolist()
    return mx, my


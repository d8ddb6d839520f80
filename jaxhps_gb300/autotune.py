"""Autotuner for the FP32 batched products of a build + solve.

An HPS tree issues a few dozen distinct product shapes (leaf operators, each
merge level's blocks, the refinement's corrections, the down pass), fixed by
(p, q, L, number of right-hand sides).  ``tune(run)`` records the shapes that
``run()`` (typically one ``build_solver`` + ``solve``) issues, times every
kernel variant of the library on each shape (CUDA events on the current
stream, synthetic operands with the recorded strides), and stores the
fastest in the library's per-shape table, which ``gemm_batched`` consults
before its built-in rules.  ``save`` / ``load`` keep a table in a JSON file.

Variants (``hps_gemm_tune_set`` in include/jaxhps_gb300.h): 0 tcgen05
3xTF32; 1 / 2 / 3 SIMT 8x8 register tiles of 128x128 / 128x64 / 64x64;
4 / 5 / 6 64x64 tiles with K split over a 2 / 4 / 8-CTA cluster; 7 SIMT 4x4
register tiles of 64x64; 8 the warp-specialised TMA + tcgen05 3xTF32 kernel
for N <= 64 (other shapes run variant 3).  All variants compute the same product; only the
order of the FP32 additions differs.  No counterpart in the reference.
"""

from __future__ import annotations

import ctypes as C
import json
import time
from pathlib import Path
from typing import Callable, Dict, List, Tuple

import torch

from . import _native as nat

VARIANTS = {
    0: "tcgen05 3xTF32",
    1: "SIMT 8x8 tiles 128x128",
    2: "SIMT 8x8 tiles 128x64",
    3: "SIMT 8x8 tiles 64x64",
    4: "64x64 split-K x2",
    5: "64x64 split-K x4",
    6: "64x64 split-K x8",
    7: "SIMT 4x4 tiles 64x64",
    8: "TMA + tcgen05 3xTF32, warp-specialised",
}

Shape = Tuple[int, ...]   # (M, N, K, batch, lda, sA, ldb, sB, ldc, sC, ldd, sD, has_C)


def record_shapes(run: Callable[[], object]) -> List[Shape]:
    """The distinct FP32 product shapes ``run()`` issues (its products run
    with the library's current choices)."""
    lib = nat.lib()
    lib.hps_gemm_shapes(1, None, 0)
    try:
        run()
        torch.cuda.synchronize()
    finally:
        n = int(lib.hps_gemm_shapes(0, None, 0))
    buf = (C.c_longlong * (13 * max(n, 1)))()
    lib.hps_gemm_shapes(-1, buf, n)
    return [tuple(int(buf[13 * i + j]) for j in range(13)) for i in range(n)]


def _extent(rows: int, cols: int, ld: int, stride: int, batch: int) -> int:
    return (batch - 1) * stride + (rows - 1) * ld + cols if stride else (rows - 1) * ld + cols


class _Operands:
    """Synthetic operands of one recorded shape (its strides kept)."""

    def __init__(self, shape: Shape):
        M, N, K, batch, lda, sA, ldb, sB, ldc, sC, ldd, sD, has_c = shape
        self.shape = shape
        dev = torch.device("cuda", torch.cuda.current_device())
        g = torch.Generator(device=dev).manual_seed(0)
        self.A = torch.randn(_extent(M, K, lda, sA, batch), device=dev, generator=g)
        self.B = torch.randn(_extent(K, N, ldb, sB, batch), device=dev, generator=g)
        self.C = torch.randn(_extent(M, N, ldc, sC, batch), device=dev, generator=g) if has_c else None
        self.D = torch.empty(_extent(M, N, ldd, sD, batch), device=dev)
        self.alpha = (C.c_double * 2)(1.0, 0.0)
        self.beta = (C.c_double * 2)(1.0 if has_c else 0.0, 0.0)

    def call(self):
        M, N, K, batch, lda, sA, ldb, sB, ldc, sC, ldd, sD, _ = self.shape
        nat.check(nat.lib().hps_gemm_batched(nat.HPS_F32, M, N, K, self.alpha, self.A.data_ptr(), lda, sA,
                                             self.B.data_ptr(), ldb, sB, self.beta, nat.ptr(self.C), ldc, sC,
                                             self.D.data_ptr(), ldd, sD, batch, nat.stream_ptr()),
                  "hps_gemm_batched")

    def time(self, reps: int, warmup: int = 2) -> float:
        for _ in range(warmup):
            self.call()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            self.call()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps


def time_shape(shape: Shape, variants=None, reps: int = 5) -> Dict[int, float]:
    """Milliseconds per product of each variant (None: the built-in choice,
    measured with no table entry for the shape) on synthetic operands."""
    ops = _Operands(shape)
    lib = nat.lib()
    out = {}
    old = lib.hps_gemm_force_variant(-1)
    try:
        for v in (variants if variants is not None else list(VARIANTS)):
            lib.hps_gemm_force_variant(-1 if v is None else v)
            out[v] = ops.time(reps)
    finally:
        lib.hps_gemm_force_variant(old)
    nat.raise_on_tc_timeout("autotune")
    return out


def tune(run: Callable[[], object], reps: int = 5, apply: bool = True) -> dict:
    """Records the shapes of ``run()``, times every variant on each and (with
    ``apply``) stores the fastest in the library's table.  Returns a report:
    per shape the chosen variant, its time and the time of the built-in
    choice (measured with no table entry)."""
    t0 = time.perf_counter()
    shapes = record_shapes(run)
    lib = nat.lib()
    report = {"shapes": [], "seconds": 0.0}
    for sh in shapes:
        M, N, K, batch = sh[:4]
        lib.hps_gemm_tune_set(M, N, K, batch, -1)
        times = time_shape(sh, [None] + list(VARIANTS), reps=reps)
        builtin = times.pop(None)
        best = min(times, key=times.get)
        if apply:
            lib.hps_gemm_tune_set(M, N, K, batch, best)
        report["shapes"].append({"M": M, "N": N, "K": K, "batch": batch, "variant": best,
                                 "variant_name": VARIANTS[best], "ms": times[best], "builtin_ms": builtin,
                                 "all_ms": {str(k): v for k, v in times.items()}})
    report["seconds"] = time.perf_counter() - t0
    report["builtin_total_ms"] = sum(s["builtin_ms"] for s in report["shapes"])
    report["tuned_total_ms"] = sum(s["ms"] for s in report["shapes"])
    return report


def table(report: dict) -> List[Tuple[int, int, int, int, int]]:
    return [(s["M"], s["N"], s["K"], s["batch"], s["variant"]) for s in report["shapes"]]


def apply_table(entries) -> None:
    lib = nat.lib()
    for M, N, K, batch, v in entries:
        nat.check(lib.hps_gemm_tune_set(int(M), int(N), int(K), int(batch), int(v)), "hps_gemm_tune_set")


def clear() -> None:
    nat.lib().hps_gemm_tune_clear()


def save(report: dict, path) -> None:
    Path(path).write_text(json.dumps({"entries": table(report), "report": report}, indent=1))


def load(path) -> None:
    apply_table(json.loads(Path(path).read_text())["entries"])

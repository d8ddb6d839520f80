"""Optional CUDA-event marks at the phase boundaries of build_solver and
solve (coefficient upload, build, boundary upload, refinement, result copy),
for reports of where an end-to-end call spends its time.  Disabled unless a
caller enables it; when enabled each mark records one event on the current
stream (no synchronisation), and copies on side streams record their own
start/end pair.

Optional NVTX ranges around the stages (``build_solver``, ``solve``, the
leaf stage, each merge and down-pass level, each refinement correction), so
a profiler's timeline and its range filters name them.  Off unless the
environment sets ``HPS_NVTX=1`` or a caller calls ``enable_nvtx()``: a
profiler filter on an enclosing range of the caller's own then sees the
same range stack as without them.  No counterpart in the reference (its
examples time whole calls with ``timeit``).
"""

from __future__ import annotations

import contextlib
import functools
import os

import torch

_nvtx = os.environ.get("HPS_NVTX", "0") not in ("", "0")

_marks = None
_side = None


def enable() -> None:
    global _marks, _side
    _marks, _side = [], []


def disable() -> None:
    global _marks, _side
    _marks, _side = None, None


def enabled() -> bool:
    return _marks is not None


def mark(name: str) -> None:
    if _marks is None:
        return
    e = torch.cuda.Event(enable_timing=True)
    e.record()
    _marks.append((name, e))


def side(name: str, start: torch.cuda.Event, end: torch.cuda.Event) -> None:
    """A copy on another stream, bracketed by events recorded on that stream."""
    if _side is not None:
        _side.append((name, start, end))


def collect() -> dict:
    """Milliseconds between consecutive marks (keyed by the later mark) and of
    each side-stream copy; clears the marks.  Synchronises the device."""
    global _marks, _side
    if _marks is None:
        return {}
    torch.cuda.synchronize()
    out = {}
    for (_, a), (name, b) in zip(_marks[:-1], _marks[1:]):
        out[name] = out.get(name, 0.0) + a.elapsed_time(b)
    for name, a, b in _side:
        out[name + " (side stream)"] = out.get(name + " (side stream)", 0.0) + a.elapsed_time(b)
    _marks, _side = [], []
    return out


def enable_nvtx(on: bool = True) -> None:
    global _nvtx
    _nvtx = bool(on)


def nvtx_enabled() -> bool:
    return _nvtx


@contextlib.contextmanager
def nvtx(name: str):
    """An NVTX push/pop range named ``name`` around the body, when enabled."""
    if not _nvtx:
        yield
        return
    torch.cuda.nvtx.range_push(name)
    try:
        yield
    finally:
        torch.cuda.nvtx.range_pop()


def ranged(name: str):
    """Decorator: the function's calls run inside ``nvtx(name)``."""
    def deco(fn):
        @functools.wraps(fn)
        def wrapper(*args, **kwargs):
            with nvtx(name):
                return fn(*args, **kwargs)
        return wrapper
    return deco

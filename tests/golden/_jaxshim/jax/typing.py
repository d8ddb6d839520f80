"""``jax.typing`` (test infrastructure; see ``jax/__init__.py``)."""

from typing import Any

DTypeLike = Any
ArrayLike = Any

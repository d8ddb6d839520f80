"""``jax.tree`` (test infrastructure; see ``jax/__init__.py``)."""

from .tree_util import tree_flatten as flatten, tree_leaves as leaves, tree_map as map  # noqa: F401

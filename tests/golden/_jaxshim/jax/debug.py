"""``jax.debug`` (test infrastructure; see ``jax/__init__.py``)."""


def print(fmt, *args, **kwargs):  # noqa: A001
    __builtins__["print"](fmt.format(*args, **kwargs)) if isinstance(__builtins__, dict) else None

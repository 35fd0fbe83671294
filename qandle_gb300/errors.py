"""Error types of the front end (mirrors qandle/errors.py:1-6)."""


class UnbuiltGateError(ValueError):
    """Raised when a gate is used before it is built (build it, or use it in a
    Circuit, which builds it)."""

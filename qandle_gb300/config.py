"""Module-level settings (mirrors qandle/config.py:3).

DEFAULT_MAPPING is the remapping used when a gate is built without an
explicit ``remapping`` argument.
"""
from . import remap

DEFAULT_MAPPING = remap.tanh

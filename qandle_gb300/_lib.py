"""Loader of the CUDA library (libqandle_gb300.so) through its C ABI.

There is no CPU fallback: if the library cannot be loaded, or a tensor is not
a CUDA tensor, the call raises.  The library is built in-tree by
qandle_gb300/build.py (``__graft_entry__.build()`` runs it).
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

from . import build as _build

_lock = threading.Lock()
_lib = None

c_void_p, c_int, c_int64, c_char_p = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_char_p
c_double, c_float = ctypes.c_double, ctypes.c_float

# name -> (restype, argtypes)
SIGNATURES = {
    "qg_version": (c_int, []),
    "qg_last_error": (c_char_p, []),
    "qg_apply_rotation": (c_int, [c_void_p, c_int64, c_int, c_int, c_int, c_void_p, c_int64, c_int, c_void_p]),
    "qg_apply_matrix": (c_int, [c_void_p, c_int64, c_int, c_int, c_void_p, c_int, c_void_p]),
    "qg_apply_cnot": (c_int, [c_void_p, c_int64, c_int, c_int, c_int, c_void_p]),
    "qg_apply_cz": (c_int, [c_void_p, c_int64, c_int, c_int, c_int, c_void_p]),
    "qg_apply_swap": (c_int, [c_void_p, c_int64, c_int, c_int, c_int, c_void_p]),
    "qg_angle_embedding_scratch_bytes": (c_int64, [c_int64, c_int]),
    "qg_angle_embedding": (c_int, [c_void_p, c_void_p, c_int64, c_int64, c_int, c_void_p, c_int, c_int,
                                   c_void_p, c_int64, c_void_p]),
    "qg_probs": (c_int, [c_void_p, c_void_p, c_int64, c_void_p]),
    "qg_probs_backward": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p]),
    "qg_measure_p0_scratch_bytes": (c_int64, [c_int64, c_int]),
    "qg_measure_p0": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p, c_int64, c_void_p]),
    "qg_measure_p0_backward": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int, c_void_p]),
    "qg_rotation_grad_scratch_bytes": (c_int64, [c_int64, c_int]),
    "qg_rotation_grad": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int, c_int, c_int, c_int,
                                 c_void_p, c_int64, c_void_p]),
}


def lib_path() -> str:
    return _build.LIB


def load():
    """Load (building first if needed) and return the ctypes library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            _build.build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name, None)
            if fn is None:
                raise RuntimeError(f"{path} does not export {name}: rebuild the library")
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc: int) -> None:
    if rc != 0:
        msg = load().qg_last_error().decode(errors="replace")
        raise RuntimeError(f"qandle_gb300 CUDA library error {rc}: {msg}")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))


def stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def require_cuda_state(state: torch.Tensor, what: str = "state") -> None:
    if not state.is_cuda:
        raise RuntimeError(f"qandle_gb300 runs on CUDA tensors only; {what} is on {state.device} "
                           "(move the circuit and its inputs with .to('cuda'))")
    if state.dtype != torch.complex64:
        raise RuntimeError(f"{what} must be complex64 (torch.cfloat), got {state.dtype}")

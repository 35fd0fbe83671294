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



class Gate(ctypes.Structure):
    """qg_gate (include/qandle_gb300.h)."""
    _fields_ = [(f, ctypes.c_int32) for f in ("kind", "q0", "q1", "src", "idx", "aux")]


class PlanOptions(ctypes.Structure):
    """qg_plan_options."""
    _fields_ = [(f, ctypes.c_int32) for f in ("tile_bits", "low_bits", "max_high", "measure",
                                              "keep_state", "segments", "reg_bits", "reg_search",
                                              "bwd_max_grad", "fwd_max_mats")]


class ProgramInfo(ctypes.Structure):
    """qg_program_info_t."""
    _fields_ = [(f, ctypes.c_int32) for f in (
        "num_qubits", "gates", "forward_passes", "backward_passes", "forward_ops", "backward_ops",
        "nparams", "ncols", "numats", "grad_slots", "forward_shared_slots", "forward_sample_slots",
        "backward_shared_slots", "backward_sample_slots", "segments", "has_embedding")] + [
        ("table_bytes", ctypes.c_int64), ("summary", ctypes.c_char * 256)]


class PassInfo(ctypes.Structure):
    """qg_pass_info_t."""
    _fields_ = [("tile_bits", ctypes.c_int32), ("nq_tile", ctypes.c_int32),
                ("run_bits", ctypes.c_int32), ("nfixed", ctypes.c_int32),
                ("gbit", ctypes.c_int32 * 16), ("fixed_gbit", ctypes.c_int32 * 32)] + [
        (f, ctypes.c_int32) for f in ("op_count", "init", "epi")] + [
        ("init_map", ctypes.c_int32 * 3)] + [
        (f, ctypes.c_int32) for f in ("ckpt", "psi_from_ckpt", "grad_base", "ngrad")] + [
        ("ops", ctypes.POINTER(ctypes.c_int32))]


class Job(ctypes.Structure):
    """qg_job."""
    _fields_ = [("prog", ctypes.c_void_p), ("table", ctypes.c_void_p), ("workspace", ctypes.c_void_p),
                ("workspace_bytes", ctypes.c_int64), ("state", ctypes.c_void_p), ("batch", ctypes.c_int64),
                ("pass_", ctypes.c_int32), ("zero_init", ctypes.c_int32), ("out", ctypes.c_void_p)]


MAX_JOBS = 32

GATE = {"rx": 0, "ry": 1, "rz": 2, "u": 3, "cnot": 4, "cz": 5, "swap": 6, "emb": 7}
MEASURE = {"none": 0, "state": 1, "probs": 2, "p0": 3, "z": 4}

# name -> (restype, argtypes)
SIGNATURES = {
    "qg_version": (c_int, []),
    "qg_last_error": (c_char_p, []),
    "qg_apply_rotation": (c_int, [c_void_p, c_int64, c_int, c_int, c_int, c_void_p, c_int64, c_int, c_void_p]),
    "qg_apply_matrix": (c_int, [c_void_p, c_int64, c_int, c_int, c_void_p, c_int, c_void_p]),
    "qg_apply_cnot": (c_int, [c_void_p, c_int64, c_int, c_int, c_int, c_void_p]),
    "qg_apply_controlled_rotation": (c_int, [c_void_p, c_int64, c_int, c_int, c_int, c_int, c_void_p, c_int64,
                                             c_int, c_void_p]),
    "qg_apply_controlled_matrix": (c_int, [c_void_p, c_int64, c_int, c_int, c_int, c_void_p, c_int, c_void_p]),
    "qg_reset": (c_int, [c_void_p, c_int64, c_int, c_int, c_void_p]),
    "qg_amplitude_embedding_scratch_bytes": (c_int64, [c_int64, c_int64]),
    "qg_amplitude_embedding": (c_int, [c_void_p, c_void_p, c_int64, c_int64, c_int, c_int64, ctypes.c_float, c_int,
                                       c_void_p, c_int64, c_void_p]),
    "qg_controlled_rotation_grad": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int, c_int, c_int, c_int,
                                            c_int, c_void_p, c_int64, c_void_p]),
    "qg_apply_cz": (c_int, [c_void_p, c_int64, c_int, c_int, c_int, c_void_p]),
    "qg_apply_swap": (c_int, [c_void_p, c_int64, c_int, c_int, c_int, c_void_p]),
    "qg_angle_embedding_scratch_bytes": (c_int64, [c_int64, c_int]),
    "qg_angle_embedding": (c_int, [c_void_p, c_void_p, c_int64, c_int64, c_int, c_void_p, c_int, c_int,
                                   c_void_p, c_int64, c_void_p]),
    "qg_probs": (c_int, [c_void_p, c_void_p, c_int64, c_void_p]),
    "qg_probs_backward": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p]),
    "qg_measure_p0_scratch_bytes": (c_int64, [c_int64, c_int]),
    "qg_measure_p0": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p, c_int64, c_void_p]),
    "qg_measure_p0_noalloc": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p]),
    "qg_measure_p0_backward": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int, c_void_p]),
    "qg_rotation_grad_scratch_bytes": (c_int64, [c_int64, c_int]),
    "qg_rotation_grad": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int, c_int, c_int, c_int,
                                 c_void_p, c_int64, c_void_p]),
    "qg_plan_options_default": (None, [ctypes.POINTER(PlanOptions)]),
    "qg_program_create": (c_int, [ctypes.POINTER(Gate), c_int, c_void_p, c_int,
                                  ctypes.POINTER(PlanOptions), ctypes.POINTER(c_void_p)]),
    "qg_program_destroy": (None, [c_void_p]),
    "qg_program_compile": (c_int, [c_void_p, c_int]),
    "qg_program_compiled": (c_int, [c_void_p]),
    "qg_program_pass_source": (c_int64, [c_void_p, c_int, c_int, c_void_p, c_int64]),
    "qg_program_info": (c_int, [c_void_p, ctypes.POINTER(ProgramInfo)]),
    "qg_program_pass": (c_int, [c_void_p, c_int, c_int, ctypes.POINTER(PassInfo)]),
    "qg_program_table": (c_int, [c_void_p, c_void_p, c_int64]),
    "qg_program_slots": (c_int, [c_void_p, c_int, c_void_p, c_int64]),
    "qg_program_grad_targets": (c_int, [c_void_p, c_void_p, c_int64]),
    "qg_program_workspace_bytes": (c_int64, [c_void_p, c_int64, c_int]),
    "qg_program_forward": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int,
                                   c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "qg_program_forward_timed": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int,
                                         c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                         c_void_p]),
    "qg_program_prepare": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int64, c_void_p, c_void_p,
                                   c_void_p, c_void_p]),
    "qg_jobs_run_pass": (c_int, [ctypes.POINTER(Job), c_int, c_void_p]),
    "qg_job_run_pass_compiled": (c_int, [ctypes.POINTER(Job), c_void_p]),
    "qg_workspace_status": (c_int, [c_void_p, c_void_p]),
    "qg_selftest_wait_timeout": (c_int, [c_int64, c_void_p]),
    "qg_fp32_probe_blocks": (c_int64, []),
    "qg_fp32_probe": (c_int, [c_void_p, c_int64, c_int64, c_void_p, c_void_p]),
    "qg_program_finish": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int64, c_void_p, c_void_p]),
    "qg_program_backward": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_int64,
                                    c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p]),
    "qg_program_backward_timed": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_int64,
                                          c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                          c_void_p, c_void_p, c_void_p, c_void_p]),
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
        # compiled pass kernels are kept on disk beside the library unless the
        # caller chose another place (an empty value turns the cache off)
        if "QG_JIT_CACHE_DIR" not in os.environ:
            cache = os.path.join(os.path.dirname(path), "jit_cache")
            try:
                os.makedirs(cache, exist_ok=True)
                os.environ["QG_JIT_CACHE_DIR"] = cache
            except OSError:
                pass
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

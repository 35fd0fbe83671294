"""Autotuner for the fused engine's plan options.

The best plan depends on the circuit and the batch:

* tile shape: a 2^13 tile holds more qubits per pass (fewer HBM round
  trips), a 2^12 tile runs two CTAs per SM, longer contiguous runs
  (``low_bits``) make the loads denser but leave fewer tile slots for strided
  qubits, and 16 instead of 32 amplitudes per thread trade exchanges for
  occupancy;
* fusion width k (``max_high``): the strided qubits a pass may take; a
  smaller k gives lighter passes (and more of them);
* qubit-remap schedule (``reg_search``): which tile qubits each exchange
  brings into the registers -- the greedy set the next gates ask for, or the
  set (searched over all of them) that places the most gates;
* pass length (``fwd_max_mats``): the 2x2 slots a pass may hold (default 24);
  longer passes make fewer HBM round trips but their unrolled code leaves
  the instruction cache.

``autotune`` plans and runs candidates on the device with the circuit's own
structure at the given batch and times each forward with CUDA events.
Without an explicit candidate list it searches in stages: the tile shapes
first, then k one and two below the tile's limit on the best shape, then the
searched remap schedule on the best of those, then pass lengths of 16 and 32
2x2 slots and uncapped passes on the best so far.  Results are kept in a JSON
file keyed by the circuit's gate structure (gate kinds and qubits, not
angles), the batch, the device and whether passes are compiled, so a later
process gets the answer without running anything.
"""
from __future__ import annotations

import hashlib
import json
import os
import threading
import typing

import torch

from . import engine

# stage 1 of the search: tile shapes (k at the tile's limit, greedy remap)
DEFAULT_CANDIDATES: typing.List[dict] = [
    dict(tile_bits=13, low_bits=6, reg_bits=5),
    dict(tile_bits=12, low_bits=6, reg_bits=5),
    dict(tile_bits=12, low_bits=7, reg_bits=5),
    dict(tile_bits=13, low_bits=7, reg_bits=5),
    dict(tile_bits=12, low_bits=6, reg_bits=4),
    dict(tile_bits=13, low_bits=6, reg_bits=4),
]


# fwd_max_mats that plans passes as long as the tile allows (a small state
# pays per pass in latency, not in HBM traffic)
UNCAPPED = 1 << 30


def _k_candidates(best: dict, n: int) -> typing.List[dict]:
    """Stage 2: k (max_high) one and two below the tile's strided limit."""
    limit = min(n, best["tile_bits"]) - min(best["low_bits"], n)
    return [dict(best, max_high=k) for k in (limit - 1, limit - 2) if k >= 1]


_lock = threading.Lock()


def default_cache_path() -> str:
    env = os.environ.get("QG_TUNE_CACHE")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "tune_cache.json")


def structure_key(lowered: "engine.Lowered") -> str:
    """Hash of what the plan depends on: width, measurement, and per gate its
    kind, qubits and whether its angle is per sample.  Angle values and
    matrix entries do not change the plan."""
    h = hashlib.sha256()
    h.update(f"n={lowered.n};m={lowered.measure};".encode())
    for g in lowered.gates:  # (kind, q0, q1, src, idx, aux); aux marks diagonal U
        kind, q0, q1, src, aux = g[0], g[1], g[2], g[3], g[5]
        h.update(f"{kind},{q0},{q1},{src},{aux};".encode())
    h.update(("q" + ",".join(str(q) for q in lowered.qlist)).encode())
    return h.hexdigest()[:32]


def _key(lowered, batch: int, device, compiled: bool) -> str:
    name = torch.cuda.get_device_name(device) if torch.cuda.is_available() else "cpu"
    return f"{structure_key(lowered)}|B={batch}|{name}|{'compiled' if compiled else 'interpreted'}"


def _load(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path: str, key: str, entry: dict) -> None:
    with _lock:
        data = _load(path)
        data[key] = entry
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        tmp = f"{path}.tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def time_candidate(circuit, batch: int, device, options: dict, reps: int = 3, compiled: bool = True) -> float:
    """Milliseconds of one forward of `circuit` at `batch` with the plan
    `options` (inputs resident on the device, after one warm-up).  Angles,
    matrices and named inputs stay zero: the kernels' work does not depend on
    their values."""
    ex = engine.FusedExecutor(circuit, compiled=compiled, **options)
    bound = engine.BoundForward(ex, batch, device)
    bound.launch()
    torch.cuda.synchronize(device)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        bound.launch()
    e1.record()
    torch.cuda.synchronize(device)
    return e0.elapsed_time(e1) / reps


def autotune(circuit, batch: int, device="cuda", candidates: typing.Optional[typing.List[dict]] = None,
             cache_path: typing.Optional[str] = None, reps: int = 3, compiled: bool = True,
             timer: typing.Optional[typing.Callable[[dict], float]] = None) -> dict:
    """Fastest plan options for `circuit` (a qandle_gb300.Circuit or its
    built UnsplittedCircuit) at `batch` on `device`.

    Returns {"options": {...}, "ms": best time, "timings": [(options, ms)],
    "cached": bool}.  Candidates that the planner rejects for this circuit
    are skipped.  `timer` replaces the device timing (tests)."""
    built = getattr(circuit, "circuit", circuit)
    if built.num_qubits < 5:  # runs on the per-gate kernels: nothing to tune
        return {"options": {}, "ms": None, "timings": [], "cached": False}
    lowered = engine.lower(built)
    device = torch.device(device)
    path = cache_path or default_cache_path()
    key = _key(lowered, batch, device, compiled)
    hit = _load(path).get(key)
    if hit is not None:
        return dict(hit, cached=True)
    timings = []

    def run(opts):
        for opt in opts:
            if any(o == opt for o, _ in timings):
                continue
            try:
                ms = timer(opt) if timer is not None else time_candidate(built, batch, device, opt, reps, compiled)
            except RuntimeError:
                continue
            timings.append((dict(opt), float(ms)))

    if candidates:
        run(candidates)
    else:
        run(DEFAULT_CANDIDATES)
        if timings:
            run(_k_candidates(min(timings, key=lambda t: t[1])[0], built.num_qubits))
            run([dict(min(timings, key=lambda t: t[1])[0], reg_search=1)])
            run([dict(min(timings, key=lambda t: t[1])[0], fwd_max_mats=m) for m in (16, 32, UNCAPPED)])
    if not timings:
        raise RuntimeError("no candidate plan could be run for this circuit")
    best = min(timings, key=lambda t: t[1])
    entry = {"options": best[0], "ms": best[1], "timings": timings}
    _store(path, key, entry)
    return dict(entry, cached=False)

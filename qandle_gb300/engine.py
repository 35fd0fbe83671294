"""Fused engine: lowering of built layers to a gate program, and the
autograd Function that runs it forward (fused passes) and backward (adjoint).

The lowering reads the same attributes the reference's built modules carry
(qandle/operators.py:215-238 BuiltParametrizedOperator .qubit/.theta/
.remapping/.named/.name, :87-104 BuiltU .qubit/.original_matrix, :536-545
BuiltCNOT .c/.t, :570-579 BuiltCZ, :653-659 BuiltSWAP .a/.b,
embeddings.py:114-137 AngleEmbeddingBuilt .qubits/.rotation/.name,
measurements.py:73-123), so a circuit of either qandle's or this package's
layer classes lowers the same way.  Unknown layers raise: there is no silent
fallback.
"""
from __future__ import annotations

import collections
import ctypes
import os
import threading
import warnings

import numpy as np
import torch
from torch.autograd.function import once_differentiable

from . import _lib

_AXIS = {"BuiltRX": 0, "BuiltRY": 1, "BuiltRZ": 2}
_MEAS = {"MeasureProbabilityBuilt": "p0", "MeasureAllAbsolute": "probs", "MeasureState": "state",
         "MeasureExpectationZBuilt": "z"}
_ROT = {"x": 0, "y": 1, "z": 2}


def _rot_axis(rotation: str) -> int:
    r = rotation.lower().replace("r", "")
    if r not in _ROT:
        raise ValueError(f"Unknown rotation {rotation}")
    return _ROT[r]


class NotFusible(ValueError):
    """A layer the fused engine knows but does not fuse (Reset, controlled
    arbitrary 2x2, multi-qubit controlled targets): the circuit runs on the
    per-gate kernels instead."""


_H = torch.tensor([[1.0, 1.0], [1.0, -1.0]], dtype=torch.complex64) / (2.0 ** 0.5)


class Lowered:
    """Gate records plus where each runtime value comes from."""

    def __init__(self, num_qubits: int):
        self.n = num_qubits
        self.gates: list[tuple] = []
        self.qlist: list[int] = []
        self.param_mods: list = []        # modules whose remapped theta feeds params[i]
        self.param_scale: list = []       # params[i] = param_scale[i] * remapping(theta)
        self.named_cols: list[tuple] = []  # (kwarg name, column or None)
        self.named_scale: list = []       # named column c is scaled by named_scale[c] (default 1)
        self.umats: list[torch.Tensor] = []
        self.measure = "state"
        self.amp_embed = None  # AmplitudeEmbeddingBuilt that sets the initial state, if any

    def _rotation(self, axis: int, qubit: int, mod, scale: float = 1.0) -> None:
        if mod.named:
            self.gates.append((axis, qubit, 0, 1, len(self.named_cols), 0))
            self.named_cols.append((mod.name, None))
            self.named_scale.append(scale)
        else:
            self.gates.append((axis, qubit, 0, 0, len(self.param_mods), 0))
            self.param_mods.append(mod)
            self.param_scale.append(scale)

    def _matrix(self, qubit: int, m: torch.Tensor) -> None:
        m = torch.as_tensor(m).to(torch.complex64).reshape(2, 2)
        diag = bool(m[0, 1] == 0 and m[1, 0] == 0)
        self.gates.append((_lib.GATE["u"], qubit, 0, 0, len(self.umats), 1 if diag else 0))
        self.umats.append(m)

    def _controlled(self, mod, inverse: bool) -> None:
        """Controlled rotation by the standard decomposition (column
        convention, applied left to right): R(t/2) on the target, CNOT,
        R(-t/2), CNOT gives R(t) where the control is 1 and I elsewhere for
        RY and RZ (X R(a) X = R(-a)); RX is H CRZ(t) H on the target."""
        t = mod.t
        tname = type(t).__name__
        if tname not in _AXIS:
            raise NotFusible(f"Controlled of {tname} runs on the per-gate kernels")
        axis = _AXIS[tname]
        sgn = -1.0 if inverse else 1.0
        c, q = mod.c, t.qubit
        rot_axis = 2 if axis == 0 else axis
        if axis == 0:
            self._matrix(q, _H)
        self._rotation(rot_axis, q, t, 0.5 * sgn)
        self.gates.append((_lib.GATE["cnot"], c, q, 0, 0, 0))
        self._rotation(rot_axis, q, t, -0.5 * sgn)
        self.gates.append((_lib.GATE["cnot"], c, q, 0, 0, 0))
        if axis == 0:
            self._matrix(q, _H)

    def add_layer(self, mod) -> None:
        name = type(mod).__name__
        if self.measure != "state" or getattr(self, "_measured", False):
            raise ValueError("layers after a measurement are not supported by the fused engine")
        if name in _AXIS:
            self._rotation(_AXIS[name], mod.qubit, mod)
        elif name == "BuiltU":
            self._matrix(mod.qubit, mod.original_matrix)
        elif name == "BuiltInvert":
            t = mod.target
            tname = type(t).__name__
            if tname in _AXIS:
                self._rotation(_AXIS[tname], t.qubit, t, -1.0)  # R(a)^-1 = R(-a)
            elif tname == "BuiltU":
                self._matrix(t.qubit, torch.linalg.inv(torch.as_tensor(t.original_matrix).to(torch.complex64)))
            elif tname in ("BuiltCNOT", "BuiltCZ", "BuiltSWAP"):
                self.add_layer(t)
            elif tname == "BuiltInvert":
                self.add_layer(t.target)
            elif tname == "BuiltControlled":
                self._controlled(t, inverse=True)
            else:
                raise NotFusible(f"Invert of {tname} runs on the per-gate kernels")
        elif name == "BuiltControlled":
            self._controlled(mod, inverse=False)
        elif name == "BuiltReset":
            raise NotFusible("Reset runs on the per-gate kernels")
        elif name == "AmplitudeEmbeddingBuilt":
            # overwrites the state: earlier layers are dead; the executor
            # writes the embedded state and runs the program on it
            self.gates, self.qlist, self.umats = [], [], []
            self.param_mods, self.param_scale, self.named_cols, self.named_scale = [], [], [], []
            self.amp_embed = mod
        elif name == "BuiltCNOT":
            self.gates.append((_lib.GATE["cnot"], mod.c, mod.t, 0, 0, 0))
        elif name == "BuiltCZ":
            self.gates.append((_lib.GATE["cz"], mod.c, mod.t, 0, 0, 0))
        elif name == "BuiltSWAP":
            self.gates.append((_lib.GATE["swap"], mod.a, mod.b, 0, 0, 0))
        elif name == "AngleEmbeddingBuilt":
            self.amp_embed = None  # a later embedding overwrites it
            qs = list(mod.qubits)
            self.gates.append((_lib.GATE["emb"], _rot_axis(mod.rotation), len(qs), 1,
                               len(self.named_cols), len(self.qlist)))
            for j in range(len(qs)):
                self.named_cols.append((mod.name, j))
            self.qlist.extend(qs)
        elif name in _MEAS:
            self.measure = _MEAS[name]
            self._measured = True
        elif hasattr(mod, "applied_gates"):  # the built ansaetze
            for m in mod.applied_gates:
                self.add_layer(m)
        elif hasattr(mod, "mods"):  # the reference's built StronglyEntanglingLayer
            for m in mod.mods:
                self.add_layer(m)
        elif name == "Circuit" and hasattr(mod, "circuit"):  # a nested circuit: its layers, inline
            if mod.num_qubits != self.n:
                raise ValueError(f"a nested circuit on {mod.num_qubits} qubits inside one on {self.n}")
            self.add_layer(mod.circuit)
        elif hasattr(mod, "layers") and hasattr(mod, "num_qubits"):
            for m in mod.layers:
                self.add_layer(m)
        else:
            raise ValueError(f"the fused engine cannot lower layer {name}")


def lower(circuit) -> Lowered:
    """Lower an UnsplittedCircuit (qandle's or this package's)."""
    lo = Lowered(circuit.num_qubits)
    for mod in circuit.layers:
        lo.add_layer(mod)
    return lo


class Program:
    """A planned gate program: host handle plus device copies of its tables."""

    def __init__(self, lowered: Lowered, measure: str, keep_state: bool, tile_bits: int = 13,
                 low_bits: int = 6, max_high: int = 0, segments: int = 1, reg_bits: int = 5,
                 reg_search: int = 0, bwd_max_grad: int = 0, fwd_max_mats: int = 0):
        lib = _lib.load()
        self.n = lowered.n
        self.measure = measure
        self.keep_state = keep_state
        self.reg_bits = reg_bits
        gates = (_lib.Gate * max(1, len(lowered.gates)))()
        for i, g in enumerate(lowered.gates):
            gates[i] = _lib.Gate(*g)
        ql = (ctypes.c_int32 * max(1, len(lowered.qlist)))(*lowered.qlist)
        opt = _lib.PlanOptions()
        lib.qg_plan_options_default(ctypes.byref(opt))
        opt.tile_bits, opt.low_bits, opt.max_high = tile_bits, low_bits, max_high
        opt.measure = _lib.MEASURE[measure]
        opt.keep_state = 1 if keep_state else 0
        opt.segments = segments
        opt.reg_bits = reg_bits
        opt.reg_search = int(reg_search)
        opt.bwd_max_grad = int(bwd_max_grad)
        opt.fwd_max_mats = int(fwd_max_mats)
        handle = ctypes.c_void_p()
        _lib.check(lib.qg_program_create(gates, len(lowered.gates), ctypes.cast(ql, ctypes.c_void_p),
                                         self.n, ctypes.byref(opt), ctypes.byref(handle)))
        self.handle = handle
        self.info = _lib.ProgramInfo()
        _lib.check(lib.qg_program_info(self.handle, ctypes.byref(self.info)))
        host = (ctypes.c_uint8 * self.info.table_bytes)()
        _lib.check(lib.qg_program_table(self.handle, host, self.info.table_bytes))
        self._table_host = torch.frombuffer(bytearray(host), dtype=torch.uint8)
        self._tables = {}
        self._compiled = set()
        self._lock = threading.Lock()          # device tables
        self._compile_lock = threading.Lock()  # compiles (seconds; must not hold up table lookups)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.load().qg_program_destroy(h)
            except Exception:
                pass

    def pass_source(self, p: int, backward: bool = False) -> str:
        """CUDA source of compiled pass p (the pass's ops unrolled)."""
        lib = _lib.load()
        bw = 1 if backward else 0
        size = lib.qg_program_pass_source(self.handle, bw, p, None, 0)
        if size < 0:
            raise IndexError(f"no {'backward' if backward else 'forward'} pass {p}")
        buf = ctypes.create_string_buffer(size)
        lib.qg_program_pass_source(self.handle, bw, p, buf, size)
        return buf.value.decode()

    def compile(self, device=None, load: bool = True, backward: bool = None, background: bool = False) -> None:
        """Compile the passes into per-pass kernels (NVRTC) for ``device``:
        the forward passes, and the backward passes too when ``backward``
        (default: when the program keeps its state for a backward).  With
        ``load=False`` only check that they build (no GPU needed);
        ``background`` compiles on a quarter of the cores at a lower
        priority.  Raises RuntimeError with the compiler's log on failure."""
        lib = _lib.load()
        if backward is None:
            backward = self.keep_state
        flags = (0 if load else 1) | (2 if backward else 0) | (4 if background else 0)
        if load:
            with torch.cuda.device(device):
                _lib.check(lib.qg_program_compile(self.handle, flags))
        else:
            _lib.check(lib.qg_program_compile(self.handle, flags))

    def compiled(self, device) -> bool:
        """True when this program's compiled kernels (forward, and backward
        for a training program) are active on ``device``."""
        with torch.cuda.device(device):
            v = _lib.load().qg_program_compiled(self.handle)
        return v == 3 if self.keep_state else v >= 1

    def ensure_compiled(self, device, background: bool = False) -> None:
        key = str(device)
        if key in self._compiled:
            return
        with self._compile_lock:
            if key not in self._compiled:
                self.compile(device, background=background)
                self._compiled.add(key)

    def table(self, device) -> torch.Tensor:
        key = str(device)
        with self._lock:
            t = self._tables.get(key)
            if t is None:
                t = self._table_host.to(device)
                self._tables[key] = t
            return t

    def summary(self) -> str:
        return self.info.summary.decode()

    def passes(self, backward: bool = False):
        """Planned passes as dicts (introspection and CPU tests)."""
        lib = _lib.load()
        out = []
        count = self.info.backward_passes if backward else self.info.forward_passes
        for i in range(count):
            pi = _lib.PassInfo()
            _lib.check(lib.qg_program_pass(self.handle, 1 if backward else 0, i, ctypes.byref(pi)))
            ops = np.ctypeslib.as_array(pi.ops, shape=(pi.op_count * 4,)).reshape(-1, 4).copy() \
                if pi.op_count else np.zeros((0, 4), np.int32)
            out.append({
                "tile_bits": pi.tile_bits, "nq_tile": pi.nq_tile, "run_bits": pi.run_bits,
                "gbit": list(pi.gbit[:pi.nq_tile]), "fixed_gbit": list(pi.fixed_gbit[:pi.nfixed]),
                "ops": ops, "init": pi.init, "epi": pi.epi, "init_map": list(pi.init_map),
                "ckpt": pi.ckpt, "psi_from_ckpt": pi.psi_from_ckpt, "grad_base": pi.grad_base,
                "ngrad": pi.ngrad})
        return out

    def slots(self, backward: bool = False):
        """Matrix slots: list of (per_sample, table_index, [(kind, src, idx, dagger), ...])."""
        lib = _lib.load()
        size = lib.qg_program_slots(self.handle, 1 if backward else 0, None, 0)
        buf = (ctypes.c_int32 * max(1, size))()
        lib.qg_program_slots(self.handle, 1 if backward else 0, ctypes.cast(buf, ctypes.c_void_p), size)
        v, out, i = list(buf)[:size], [], 0
        while i < size:
            ps, ti, cl = v[i], v[i + 1], v[i + 2]
            chain = [tuple(v[i + 3 + 4 * k: i + 7 + 4 * k]) for k in range(cl)]
            out.append((ps, ti, chain))
            i += 3 + 4 * cl
        return out

    def grad_targets(self):
        """Backward gradient slots as (src, idx): src 0 = params, 1 = named column."""
        lib = _lib.load()
        count = lib.qg_program_grad_targets(self.handle, None, 0)
        buf = (ctypes.c_int32 * max(1, 2 * count))()
        lib.qg_program_grad_targets(self.handle, ctypes.cast(buf, ctypes.c_void_p), 2 * count)
        return [(buf[2 * i], buf[2 * i + 1]) for i in range(count)]

    def workspace(self, batch: int, backward: bool, device) -> torch.Tensor:
        nb = _lib.load().qg_program_workspace_bytes(self.handle, batch, 1 if backward else 0)
        if nb < 0:
            raise RuntimeError("invalid workspace query")
        return torch.empty(max(int(nb), 256), dtype=torch.uint8, device=device)


# QG_CHECK_STATUS=1: read the workspace status word after every fused forward
# and backward (one stream synchronisation per call) and raise on a timeout.
# Without it the status words are still read, without blocking (_StatusWatch).
_CHECK_STATUS = os.environ.get("QG_CHECK_STATUS", "0") not in ("", "0")


def check_status(workspace: torch.Tensor) -> None:
    """Raise RuntimeError when a pass kernel that used `workspace` reported a
    timed-out wait (its results are then invalid).  Synchronises the current
    stream."""
    _lib.check(_lib.load().qg_workspace_status(workspace.data_ptr(), _lib.stream()))


class _StatusWatch:
    """Reads the pass kernels' status words without blocking the host.

    After every fused forward or backward, the first 16 bytes of the call's
    workspace (the status word and, after a timeout, where the wait gave up)
    are copied on the same stream into a ring of pinned host slots, and an
    event marks the copy.  Each later call first looks at the
    copies that have landed (oldest first, stopping at the first still in
    flight) and raises RuntimeError for a nonzero word: a pass kernel's
    bounded wait ran out, so that earlier call's results are invalid.  The
    copy is ordered before the workspace returns to the allocator, so a later
    call that reuses the memory and clears the word cannot hide it.  Only a
    full ring (RING copies in flight) makes a call wait for the oldest."""

    RING = 64

    def __init__(self):
        self._host = None
        self._pending = collections.deque()  # (slot, event, what)
        self._free = list(range(self.RING))
        self._lock = threading.Lock()

    # where a wait gave up (the kernels' wait-site codes)
    SITES = {1: "forward producer", 2: "forward compute warps", 5: "backward producer",
             6: "backward compute warps"}

    def _take(self, slot, ev, what):
        v, site, block, tile = (int(x) for x in self._host[slot])
        self._free.append(slot)
        if v != 0:
            raise RuntimeError(f"a fused {what} reported status {v}: a pass kernel's wait timed out "
                               f"({self.SITES.get(site, site)}, block {block}, tile {tile}: a producer / "
                               "compute hand-off never completed); its results are invalid")

    def poll(self) -> None:
        with self._lock:
            while self._pending and self._pending[0][1].query():
                self._take(*self._pending.popleft())

    def record(self, workspace: torch.Tensor, what: str) -> None:
        with self._lock:
            if self._host is None:
                self._host = torch.zeros(self.RING, 4, dtype=torch.int32, pin_memory=True)
            while self._pending and self._pending[0][1].query():
                self._take(*self._pending.popleft())
            if not self._free:
                slot, ev, w = self._pending.popleft()
                ev.synchronize()
                self._take(slot, ev, w)
            slot = self._free.pop()
            self._host[slot].copy_(workspace[:16].view(torch.int32), non_blocking=True)
            ev = torch.cuda.Event()
            ev.record()
            self._pending.append((slot, ev, what))

    def drain(self) -> None:
        """Wait for every copy in flight and raise for a nonzero word."""
        with self._lock:
            while self._pending:
                slot, ev, w = self._pending.popleft()
                ev.synchronize()
                self._take(slot, ev, w)


STATUS = _StatusWatch()


def _gather_params(lo: Lowered, device) -> torch.Tensor:
    """params[i] = param_scale[i] * remapping_i(theta_i) for every unnamed
    rotation, as one float32 vector on `device`.  The thetas are stacked by
    one op and each remapping (an elementwise function) runs once on the
    angles that use it, so a call costs a handful of ops, not a few per gate;
    gradients reach every theta through the stack."""
    mods = lo.param_mods
    thetas = [m.theta for m in mods]
    if any(t.numel() != 1 for t in thetas):
        raise ValueError("a rotation angle must hold one value")
    shape0 = thetas[0].shape
    if any(t.shape != shape0 for t in thetas):
        thetas = [t.reshape(()) for t in thetas]
    vals = torch.stack(thetas).reshape(-1)
    groups: dict = {}
    for i, m in enumerate(mods):
        groups.setdefault(m.remapping, []).append(i)
    if len(groups) == 1:
        vals = next(iter(groups))(vals)
    else:
        parts = torch.empty_like(vals)
        for fn, idx in groups.items():
            ix = torch.tensor(idx, device=vals.device)
            parts = parts.index_put((ix,), fn(vals[ix]))
        vals = parts
    vals = vals.to(device=device, dtype=torch.float32)
    scales = lo.param_scale if len(lo.param_scale) == len(mods) else None
    if scales is not None and any(sc != 1.0 for sc in scales):
        vals = vals * torch.tensor(scales, dtype=torch.float32, device=device)
    return vals.contiguous()


def _named_plan(lo: Lowered):
    """Named columns grouped by input name, in first-use order: [(name,
    [j, ...] or None)]; a name used both indexed and whole gets two groups."""
    plan = getattr(lo, "_named_plan_cache", None)
    if plan is None:
        groups: dict = {}
        for name, j in lo.named_cols:
            groups.setdefault((name, j is None), []).append(j)
        plan = [(name, None if whole else js) for (name, whole), js in groups.items()]
        # a whole (unindexed) input contributes one column per use
        plan = [(name, js) for name, js in plan for _ in range(len(groups[(name, True)]) if js is None else 1)]
        lo._named_plan_cache = plan
    return plan


def _named_order(lo: Lowered, device):
    """Permutation from the grouped column order of _named_plan to the
    column order of lo.named_cols, and the column scales (None when they are
    the identity / all one)."""
    key = ("_named_order_cache", str(device))
    cache = getattr(lo, "_named_order_cache", None)
    if cache is not None and cache[0] == key:
        return cache[1], cache[2]
    slots: dict = {}
    pos = 0
    for name, js in _named_plan(lo):
        if js is None:
            slots.setdefault((name, None), []).append(pos)
            pos += 1
        else:
            for j in js:
                slots.setdefault((name, j), []).append(pos)
                pos += 1
    used: dict = {}
    perm = []
    for name, j in lo.named_cols:
        k = used.get((name, j), 0)
        perm.append(slots[(name, j)][k])
        used[(name, j)] = k + 1
    perm_t = None if perm == list(range(len(perm))) else torch.tensor(perm, device=device)
    sc = list(lo.named_scale) + [1.0] * (len(lo.named_cols) - len(lo.named_scale))
    scale_t = None if all(x == 1.0 for x in sc) else torch.tensor(sc, dtype=torch.float32, device=device)
    lo._named_order_cache = (key, perm_t, scale_t)
    return perm_t, scale_t


class _Inputs:
    """Runtime values of one call, gathered on the device."""

    def __init__(self, lo: Lowered, state, kwargs, device):
        sizes = []
        if state is not None and state.dim() == 2:
            sizes.append(state.shape[0])
        # one block per named input: its columns (v[..., j] for an indexed
        # input, v itself otherwise) gathered by one op
        blocks = []
        for name, idx in _named_plan(lo):
            if name not in kwargs:
                raise KeyError(f"missing named input {name!r}")
            v = torch.as_tensor(kwargs[name]).to(device=device, dtype=torch.float32)
            if idx is None:
                blk = v.unsqueeze(-1)
            else:
                if v.dim() == 0:
                    raise ValueError(f"named input {name!r} is indexed per qubit but is a scalar")
                blk = v.index_select(-1, torch.as_tensor(idx, device=v.device))
            if blk.dim() > 2:
                raise ValueError(f"named input {name!r} must be a scalar or [batch] per gate")
            if blk.dim() == 2:
                sizes.append(blk.shape[0])
            blocks.append(blk)
        big = [s for s in sizes if s != 1]
        if big and any(s != big[0] for s in big):
            raise ValueError(f"inconsistent batch sizes {sizes}")
        self.batch = big[0] if big else (1 if not sizes else sizes[0])
        self.unbatched = not sizes
        if blocks:
            named = torch.cat([b.expand(self.batch, -1) if b.dim() == 2 else b.unsqueeze(0).expand(self.batch, -1)
                               for b in blocks], 1)
            perm, scale = _named_order(lo, device)
            if perm is not None:
                named = named.index_select(1, perm)
            if scale is not None:
                named = named * scale
            self.named = named.contiguous()
        else:
            self.named = torch.zeros(1, 1, dtype=torch.float32, device=device)
        if lo.param_mods:
            self.params = _gather_params(lo, device)
        else:
            self.params = torch.zeros(1, dtype=torch.float32, device=device)
        if lo.umats:
            # the lowering holds its own copies of the fixed matrices, so the
            # stacked table moves to a device once
            cache = lo.__dict__.setdefault("_umats_dev", {})
            key = str(device)
            if key not in cache:
                cache[key] = torch.stack(lo.umats).to(device).contiguous()
            self.umats = cache[key]
        else:
            self.umats = torch.zeros(1, 2, 2, dtype=torch.complex64, device=device)


_SM_COUNT: dict = {}


def _sm_count(device: torch.device) -> int:
    idx = device.index if device.index is not None else torch.cuda.current_device()
    if idx not in _SM_COUNT:
        _SM_COUNT[idx] = torch.cuda.get_device_properties(idx).multi_processor_count
    return _SM_COUNT[idx]


def _out_shape(measure, out, n, unbatched):
    if measure in ("p0", "z"):
        return out.transpose(0, 1).squeeze().transpose(-1, 0)
    if unbatched:
        return out.reshape(1 << n)
    return out


def _event_handles(events):
    """cudaEvent_t handles of torch CUDA events, as a ctypes array (torch
    creates an event's handle at its first record, so unrecorded events are
    recorded once on the current stream first)."""
    for e in events:
        if not e.cuda_event:
            e.record()
    return (ctypes.c_void_p * len(events))(*[e.cuda_event for e in events])


class _FusedRun(torch.autograd.Function):
    # grad mode is off inside forward: the caller decides whether to keep the
    # final state for the backward (`prog` is the training or inference plan)
    @staticmethod
    def forward(ctx, ex, prog, state_in, params, named, umats, batch, zero_init):
        return ex.run_forward(ctx, prog, state_in, params, named, umats, batch, zero_init)

    @staticmethod
    @once_differentiable
    def backward(ctx, gout):
        return (None,) + ctx.ex.run_backward(ctx, gout)


class FusedExecutor:
    """Runs a built circuit through the fused engine (used by Circuit)."""

    # inference calls keep at most this many captured forwards (one per
    # device, batch and input kind), least recently used dropped first
    MAX_GRAPHS = 2

    def __init__(self, circuit, tile_bits: int = 13, low_bits: int = 6, max_high: int = 0,
                 checkpoint_segments: int = 1, reg_bits: int = 5, compiled: bool = None,
                 graphs: bool = None, reg_search: int = 0, bwd_max_grad: int = 0, fwd_max_mats: int = 0):
        self.circuit = circuit
        # graphs = True: an inference call (no gradient needed, a measured
        # output) replays one captured CUDA graph of the whole forward, kept
        # per (device, batch, input kind); the default follows QG_GRAPHS (on
        # unless set to 0)
        if graphs is None:
            graphs = os.environ.get("QG_GRAPHS", "1") != "0"
        self.graphs = bool(graphs)
        self._bounds = collections.OrderedDict()
        self._bounds_lock = threading.Lock()
        # compiled = True: forward passes run as per-program kernels compiled
        # at first use (NVRTC); False: the prebuilt op interpreter.  The
        # default follows QG_COMPILE (on unless set to 0).
        if compiled is None:
            compiled = os.environ.get("QG_COMPILE", "1") != "0"
        self.compiled = bool(compiled)
        self.n = circuit.num_qubits
        try:
            self.lowered = lower(circuit)
            self.fusible = True
        except NotFusible as e:
            # the circuit holds a layer the fused engine does not fuse: it
            # runs on the per-gate kernels (same library, one launch per gate)
            self.lowered = None
            self.fusible = False
            warnings.warn(f"{e}; this circuit runs one kernel per gate")
        self.options = dict(tile_bits=tile_bits, low_bits=low_bits, max_high=max_high, reg_bits=reg_bits,
                            reg_search=int(reg_search), bwd_max_grad=int(bwd_max_grad),
                            fwd_max_mats=int(fwd_max_mats))
        self.checkpoint_segments = checkpoint_segments
        self._programs = {}  # (training, uncapped passes) -> Program
        self._last_long: dict = {}
        # timing hook: a list of 2 x (backward passes) CUDA events makes the
        # next backward record a pair around every backward pass (then clears)
        self.backward_events = None

    def program(self, training: bool, batch: int = None, device=None) -> Program:
        """The planned program for inference or training.  With the pass
        length left at its default, a call whose passes have fewer tiles than
        the device has SMs gets the plan with uncapped forward passes: such a
        pass does not fill the GPU, so it costs a tile's latency, and fewer,
        longer passes are faster.  Without `batch`, the plan the last call
        with this `training` used (the default plan before any call)."""
        training = bool(training)
        if batch is None:
            long = self._last_long.get(training, False)
        else:
            long = self.options.get("fwd_max_mats", 0) == 0 and self._small(batch, device)
            self._last_long[training] = long
        key = (training, long)
        p = self._programs.get(key)
        if p is None:
            opts = dict(self.options, fwd_max_mats=1 << 30) if long else self.options
            p = Program(self.lowered, self.lowered.measure, keep_state=training,
                        segments=self.checkpoint_segments if training else 1, **opts)
            self._programs[key] = p
        return p

    def _small(self, batch: int, device) -> bool:
        """True when a forward pass at `batch` has fewer tiles than `device`
        has SMs."""
        tb = self.options.get("tile_bits", 13)
        n = self.n
        tiles = batch << (n - tb) if n >= tb else -(-batch // (1 << (tb - n)))
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        return tiles < _sm_count(dev)

    def __call__(self, state=None, **kwargs):
        if self.n < 5 or not self.fusible:
            # the fused tile needs five qubits in registers; tiny circuits run the per-gate kernels
            return self.circuit.forward(state, **kwargs)
        if self.lowered.amp_embed is not None:
            state = self.lowered.amp_embed(**kwargs)  # the embedded features are the input state
        dev = state.device if state is not None else self._device(kwargs)
        if dev.type != "cuda":
            raise RuntimeError("qandle_gb300 runs on CUDA tensors only; move the circuit and its inputs "
                               "with .to('cuda')")
        if state is not None:
            _lib.require_cuda_state(state)
        STATUS.poll()
        inp = _Inputs(self.lowered, state, kwargs, dev)
        zero_init = 1 if (state is None and not self._has_embedding()) else 0
        training = torch.is_grad_enabled() and any(
            t is not None and t.requires_grad for t in (state, inp.params, inp.named))
        if not training and self.graphs and self.lowered.measure != "state":
            out = self._replay(inp, state, dev)
            return _out_shape(self.lowered.measure, out, self.n, inp.unbatched)
        out = _FusedRun.apply(self, self.program(training, inp.batch, dev), state, inp.params, inp.named, inp.umats,
                              inp.batch, zero_init)
        return _out_shape(self.lowered.measure, out, self.n, inp.unbatched)

    def _replay(self, inp: "_Inputs", state, dev) -> torch.Tensor:
        """Inference through a captured forward: the call's values go into the
        static buffers of a BoundForward for (device, batch, whether a state
        is given), captured into one CUDA graph at its first use, and the
        graph is replayed on the current stream.  Returns a copy of the
        measured output (the static output buffer is reused by the next
        call)."""
        key = (str(dev), inp.batch, state is not None)
        with self._bounds_lock:
            b = self._bounds.pop(key, None)
            if b is None:
                while len(self._bounds) >= self.MAX_GRAPHS:
                    self._bounds.popitem(last=False)
                b = BoundForward(self, inp.batch, dev, has_state=state is not None)
            self._bounds[key] = b
        b.set_from(inp, state)
        if b.graph is None:
            b.capture()
            if state is not None:
                # the capture's warm-up launch ran the forward on the static
                # buffers, and a plan of several passes stores its state
                # between passes in place: the call's input state goes in again
                b.set_from(inp, state)
        b.replay()  # records the status word
        if _CHECK_STATUS:
            check_status(b.ws)
        return b.out.clone()

    def _has_embedding(self) -> bool:
        return any(g[0] == _lib.GATE["emb"] for g in self.lowered.gates)

    def _device(self, kwargs):
        for v in kwargs.values():
            if isinstance(v, torch.Tensor):
                return v.device
        buf = getattr(self.circuit, "state", None)
        if isinstance(buf, torch.Tensor):
            return buf.device
        return torch.device("cpu")

    # -- forward / backward bodies (called from the autograd Function) --

    def run_forward(self, ctx, prog: Program, state_in, params, named, umats, batch, zero_init):
        n = self.n
        dev = params.device
        B = batch
        if state_in is not None and not prog.info.has_embedding:
            st = state_in.reshape(-1, 1 << n)
            st = (st.expand(B, -1) if st.shape[0] == 1 and B > 1 else st).contiguous().clone()
        else:
            st = torch.empty(B, 1 << n, dtype=torch.complex64, device=dev)
        m = prog.measure
        if m in ("p0", "z"):
            out = torch.empty(B, n, dtype=torch.float32, device=dev)
        elif m == "probs":
            out = torch.empty(B, 1 << n, dtype=torch.float32, device=dev)
        else:
            out = None
        ckpt = None
        if prog.info.segments > 1:
            ckpt = torch.empty(prog.info.segments - 1, B, 1 << n, dtype=torch.complex64, device=dev)
        ws = prog.workspace(B, False, dev)
        if self.compiled:
            prog.ensure_compiled(dev)
        _lib.call("qg_program_forward", prog.handle, prog.table(dev).data_ptr(), ws.data_ptr(), ws.numel(),
                  st.data_ptr(), B, zero_init, params.data_ptr(), named.data_ptr(), umats.data_ptr(),
                  _lib.ptr(out), _lib.ptr(ckpt), _lib.stream())
        if _CHECK_STATUS:
            check_status(ws)
        else:
            STATUS.record(ws, "forward")
        ctx.ex = self
        ctx.prog = prog
        ctx.batch = B
        ctx.state_shape = None if state_in is None else state_in.shape
        if prog.keep_state:
            ctx.save_for_backward(st, params, named, umats)
            ctx.ckpt = ckpt
        result = st if out is None else out
        return result

    def run_backward(self, ctx, gout):
        prog: Program = ctx.prog
        if not prog.keep_state:
            raise RuntimeError("the fused forward ran without gradient tracking")
        st, params, named, umats = ctx.saved_tensors
        STATUS.poll()  # a forward whose wait ran out has no valid state to differentiate
        if getattr(ctx, "_consumed", False):
            raise RuntimeError("the fused engine's backward can run once per forward "
                               "(retain_graph is not supported)")
        ctx._consumed = True
        n, B, dev = self.n, ctx.batch, st.device
        m = prog.measure
        if m in ("p0", "z", "probs"):
            g = gout.to(torch.float32).reshape(B, -1).contiguous()
        else:
            g = gout.to(torch.complex64).reshape(B, 1 << n).contiguous()
        lam = torch.empty_like(st)
        ws = prog.workspace(B, True, dev)
        dparams = torch.empty(max(1, prog.info.nparams), dtype=torch.float32, device=dev)
        dnamed = torch.empty(B, max(1, prog.info.ncols), dtype=torch.float32, device=dev)
        need_state = ctx.needs_input_grad[2] and not prog.info.has_embedding
        dstate = torch.empty_like(st) if need_state else None
        evp = None
        events = self.backward_events
        if events is not None:
            # one backward records an event pair around every backward pass
            self.backward_events = None
            evp = _event_handles(events)
        _lib.call("qg_program_backward_timed", prog.handle, prog.table(dev).data_ptr(), ws.data_ptr(), ws.numel(),
                  st.data_ptr(), lam.data_ptr(), B, params.data_ptr(), named.data_ptr(), umats.data_ptr(),
                  g.data_ptr(), dparams.data_ptr(), dnamed.data_ptr(), _lib.ptr(dstate),
                  _lib.ptr(ctx.ckpt), evp, _lib.stream())
        if _CHECK_STATUS:
            check_status(ws)
        else:
            STATUS.record(ws, "backward")
        gstate = None
        if need_state:
            shp = ctx.state_shape
            gstate = dstate
            if len(shp) == 1:
                gstate = dstate.sum(0)
            elif shp[0] != B:
                gstate = dstate.sum(0, keepdim=True)
            gstate = gstate.reshape(shp)
        gp = dparams[:params.numel()] if ctx.needs_input_grad[3] else None
        gn = dnamed[:, :named.shape[1]].reshape(named.shape) if (ctx.needs_input_grad[4] and named.dim() == 2) else None
        return None, gstate, gp, gn, None, None, None


class BoundForward:
    """Static buffers for repeated inference calls at one batch size.

    ``set_inputs`` copies a call's values into the buffers, ``launch`` runs
    the planned passes on the current stream (optionally recording an event
    pair around every pass), and ``capture``/``replay`` put the whole forward
    (matrix build, embedding factors, every pass, measurement) into one CUDA
    graph so a call costs a single graph launch.
    """

    def __init__(self, ex: "FusedExecutor", batch: int, device, has_state: bool = False):
        self.ex = ex
        self.prog = ex.program(False, batch, device)
        self.n = ex.n
        self.batch = batch
        self.device = torch.device(device)
        info = self.prog.info
        n = self.n
        self.state = torch.zeros(batch, 1 << n, dtype=torch.complex64, device=device)
        m = self.prog.measure
        if m in ("p0", "z"):
            self.out = torch.empty(batch, n, dtype=torch.float32, device=device)
        elif m == "probs":
            self.out = torch.empty(batch, 1 << n, dtype=torch.float32, device=device)
        else:
            self.out = None
        self.ws = self.prog.workspace(batch, False, device)
        self.params = torch.zeros(max(1, info.nparams), dtype=torch.float32, device=device)
        self.named = torch.zeros(batch, max(1, info.ncols), dtype=torch.float32, device=device)
        self.umats = torch.zeros(max(1, info.numats), 2, 2, dtype=torch.complex64, device=device)
        self.table = self.prog.table(device)
        self.zero_init = 0 if (has_state or info.has_embedding) else 1
        self.graph = None
        if ex.compiled:
            self.prog.ensure_compiled(self.device)

    def set_inputs(self, state=None, **kwargs) -> None:
        with torch.no_grad():
            self.set_from(_Inputs(self.ex.lowered, state, kwargs, self.device), state)

    def set_from(self, inp: "_Inputs", state=None) -> None:
        """Copy the gathered values of one call (and its input state) into
        the static buffers, on the current stream."""
        with torch.no_grad():
            if inp.batch != self.batch and inp.batch != 1:
                raise ValueError(f"bound for batch {self.batch}, got {inp.batch}")
            self.params[:inp.params.numel()].copy_(inp.params)
            if self.ex.lowered.named_cols:
                self.named.copy_(inp.named.expand(self.batch, -1))
            if self.ex.lowered.umats:
                self.umats.copy_(inp.umats)
            if state is not None:
                self.state.copy_(state.reshape(-1, 1 << self.n).expand(self.batch, -1))

    def launch(self, events=None, record_status: bool = True) -> None:
        evp = None
        if events is not None:
            evp = _event_handles(events)
        if record_status:  # (not while a graph is being captured)
            STATUS.poll()
        _lib.call("qg_program_forward_timed", self.prog.handle, self.table.data_ptr(), self.ws.data_ptr(),
                  self.ws.numel(), self.state.data_ptr(), self.batch, self.zero_init, self.params.data_ptr(),
                  self.named.data_ptr(), self.umats.data_ptr(), _lib.ptr(self.out), None, evp,
                  _lib.stream())
        if record_status:
            STATUS.record(self.ws, "forward")

    def capture(self) -> None:
        """Capture the forward into a CUDA graph.  A warm-up launch runs
        first (outside the graph), and it advances the static state buffer
        when the plan has several passes: set an input state again before
        the first replay."""
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.launch()  # warm-up outside the graph (sets kernel attributes)
        torch.cuda.current_stream(self.device).wait_stream(s)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.launch(record_status=False)

    def replay(self) -> None:
        STATUS.poll()
        self.graph.replay()
        STATUS.record(self.ws, "forward")

    def result(self) -> torch.Tensor:
        return self.state if self.out is None else self.out

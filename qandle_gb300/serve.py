"""Continuous-batching serving loop for circuit evaluations.

Requests are circuits from the strongly-entangling family (AngleEmbedding,
RZ RY RZ layers, CNOT rings, <Z> out) of 4..24 qubits and any batch.  The
loop keeps every admitted request's state, matrix tables and embedding
factors on the device and advances all admitted requests together: each
step is ONE multi-job launch of the fused pass kernel (qg_jobs_run_pass)
that runs the next pass of every active request, whatever its width, plus
one launch of its own compiled pass kernel for each large request whose
program has been compiled (in the background, once per structure).  New
requests are admitted between steps as soon as the HBM budget has room, so
requests that arrive while others are on the GPU join the running batch
instead of waiting for it to drain.  A request counts against the budget
with everything it holds on the device while admitted: its state
(2^n * 8 B * batch), its program workspace (matrix tables, embedding factors,
measurement partials) and its output.

Each request's tiles are computed by the same code in the same order
whatever else shares the launch, and its reductions run in a fixed order,
so a request's result is bit-identical alone and in the mix.  The
interpreted kernel and a program's compiled kernels run the same op list
through the same arithmetic (only the dispatch on register positions
differs), so a request that moves to the compiled kernels once they are
ready, at a pass boundary, gets the same bits as one that never does.

There is no CPU path: the loop drives the CUDA library through its C ABI.
"""
from __future__ import annotations

import collections
import concurrent.futures as cf
import ctypes
import heapq
import itertools
import threading
import time

import numpy as np
import torch

from . import _lib
from .engine import Lowered, Program

_ROT = {"rx": 0, "ry": 1, "rz": 2}


def lower_description(desc: dict, pad_to: int = 5):
    """Gate records and runtime values of a circuit description (see
    qandle_gb300.workloads).  Circuits narrower than `pad_to` qubits get idle
    qubits prepended (qubit indices shift up), which leaves <Z> of the real
    qubits unchanged; returns (lowered, params, named [B, ncols], shift)."""
    n = desc["n"]
    shift = max(0, pad_to - n)
    lo = Lowered(n + shift)
    params, cols = [], []
    inputs = desc.get("inputs", {})
    for g in desc["gates"]:
        k = g[0]
        if k == "emb":
            qs = [q + shift for q in g[3]]
            lo.gates.append((_lib.GATE["emb"], _ROT[g[1]], len(qs), 1, len(lo.named_cols), len(lo.qlist)))
            x = np.asarray(inputs[g[2]], dtype=np.float32)
            for j in range(len(qs)):
                lo.named_cols.append((g[2], j))
                cols.append(x[..., j])
            lo.qlist.extend(qs)
        elif k in _ROT:
            if g[3] is None:
                lo.gates.append((_ROT[k], g[1] + shift, 0, 0, len(params), 0))
                params.append(np.float32(g[2]))
            else:
                lo.gates.append((_ROT[k], g[1] + shift, 0, 1, len(lo.named_cols), 0))
                lo.named_cols.append((g[3], None))
                cols.append(np.asarray(inputs[g[3]], dtype=np.float32))
        elif k in ("cnot", "cz", "swap"):
            lo.gates.append((_lib.GATE[k], g[1] + shift, g[2] + shift, 0, 0, 0))
        else:
            raise ValueError(f"the serving loop does not take gate {k}")
    lo.measure = desc.get("measure", "z")
    B = desc["batch"] or 1
    named = (np.stack([np.broadcast_to(c, (B,)) for c in cols], 1).astype(np.float32)
             if cols else np.zeros((B, 1), np.float32))
    return lo, np.asarray(params + [np.float32(0)], np.float32), named, shift


def description_from_qasm(text: str, inputs: dict, batch: int, measure: str = "z") -> dict:
    """A serving request from OpenQASM 2/3 text (the wire format): rx/ry/rz
    with values or named inputs (``inputs[name]`` = [batch] angles), cx, cz,
    swap.  The measurement is <Z> unless ``measure`` says otherwise."""
    from . import operators, qasm

    layers, n = qasm.parse(text)
    gates = []
    for lay in layers:
        if isinstance(lay, operators.UnbuiltParametrizedOperator):
            k = type(lay).__name__.lower()
            if lay.named:
                gates.append((k, lay.qubit, None, lay.name))
            else:
                gates.append((k, lay.qubit, float(lay.remapping(lay.theta).detach()), None))
        elif isinstance(lay, operators.CNOT):
            gates.append(("cnot", lay.c, lay.t))
        elif isinstance(lay, operators.CZ):
            gates.append(("cz", lay.c, lay.t))
        elif isinstance(lay, operators.SWAP):
            gates.append(("swap", lay.a, lay.b))
        elif type(lay).__name__.startswith("Measure"):
            continue
        else:
            raise ValueError(f"the serving loop does not take {type(lay).__name__}")
    return {"name": "qasm", "n": n, "batch": batch, "gates": gates,
            "inputs": {k: np.asarray(v, dtype=np.float32) for k, v in inputs.items()}, "measure": measure}


def structure_key(lo: Lowered):
    return (lo.n, lo.measure, tuple(lo.gates), tuple(lo.qlist))


def _tiles_per_pass(n: int, batch: int, tile_bits: int) -> int:
    """Tiles one pass of a request walks (the pass kernels' work unit)."""
    if n >= tile_bits:
        return batch << (n - tile_bits)
    per_tile = 1 << (tile_bits - n)
    return (batch + per_tile - 1) // per_tile


class _Slot:
    __slots__ = ("req", "prog", "state", "ws", "out", "host_out", "batch", "next_pass", "bytes",
                 "event", "params", "named", "umats", "shift", "tiles", "idle", "compiled")

    def remaining(self) -> int:
        return self.tiles * (self.prog.info.forward_passes - self.next_pass)


class _CompileQueue:
    """Programs waiting for their compile, largest work first.  A program
    (by identity: the server keeps every program it planned) enters at most
    once; after close, pop returns None and queued programs are dropped."""

    def __init__(self):
        self._heap: list = []  # (-work, seq, program)
        self._seq = itertools.count()
        self._seen: set = set()
        self._cv = threading.Condition()
        self._closed = False

    def push(self, prog, work: int) -> bool:
        with self._cv:
            if self._closed or id(prog) in self._seen:
                return False
            self._seen.add(id(prog))
            heapq.heappush(self._heap, (-int(work), next(self._seq), prog))
            self._cv.notify()
            return True

    def claim(self, prog) -> None:
        """Mark a program compiled elsewhere, so that it is not queued."""
        with self._cv:
            self._seen.add(id(prog))

    def pop(self):
        with self._cv:
            while not self._heap and not self._closed:
                self._cv.wait()
            if self._closed:
                return None
            return heapq.heappop(self._heap)[2]

    def close(self) -> None:
        with self._cv:
            self._closed = True
            self._cv.notify_all()


class Request:
    def __init__(self, desc: dict, arrival: float | None = None):
        self.desc = desc
        self.arrival = time.perf_counter() if arrival is None else arrival
        self.admitted = None
        self.completed = None
        self.future: cf.Future = cf.Future()
        self.lowered = None   # (lowered, params, named, shift), set at submit
        self.prog = None
        self.need = 0         # device bytes while admitted
        self.work = 0         # tiles over all passes (the scheduling key)

    @property
    def latency(self):
        return None if self.completed is None else self.completed - self.arrival


class Server:
    """Continuous-batching executor on one device.

    hbm_budget: device bytes the admitted requests may hold together (state,
    workspace and output of each).  max_active: requests admitted at once (a
    step of more than the 32 jobs one launch takes is several launches).

    policy "srpt" (default) schedules by shortest remaining work, counted in
    pass tiles: admission takes the queued request with the least work that
    fits the budget (a request queued longer than max_queue_wait_s goes
    first), and each step advances the active requests with the least
    remaining work until the step holds step_tiles tiles (at least one
    request; a request left out for max_idle_steps steps is always taken).
    Small requests then finish in a few short steps instead of sharing every
    step with the largest ones.  policy "all" admits oldest first and
    advances every active request every step.  Either way a request's result
    does not depend on what else ran: the same kernel computes its tiles in
    the same order.

    compile_min_tiles: a request whose passes walk at least this many tiles
    has its program's passes compiled (NVRTC) on a background thread, once
    per structure, largest work first; from the first step after they are
    ready its passes run as launches of those kernels, which execute fewer
    instructions than the interpreted multi-job kernel.  Smaller requests
    share the interpreted launches.  None turns compiling off.
    """

    def __init__(self, device="cuda", hbm_budget: int = 64 << 30, max_active: int = 64,
                 tile_bits: int = 13, low_bits: int = 6, policy: str = "srpt", step_tiles: int = 1 << 16,
                 max_idle_steps: int = 64, max_queue_wait_s: float = 10.0, max_inflight_steps: int = 2,
                 planning_threads: int = 4, compile_min_tiles: int | None = 1024):
        if policy not in ("srpt", "all"):
            raise ValueError(f"policy must be 'srpt' or 'all', got {policy!r}")
        self.device = torch.device(device)
        self.budget = int(hbm_budget)
        self.max_active = max_active
        self.policy = policy
        self.step_tiles = int(step_tiles)
        self.max_idle_steps = int(max_idle_steps)
        self.max_queue_wait_s = float(max_queue_wait_s)
        self.tile_bits = tile_bits
        self.max_inflight_steps = max(1, int(max_inflight_steps))
        # passes as long as the tile allows: every pass of a request is one
        # scheduling step, and the interpreted kernel does not unroll its ops
        self.opts = dict(tile_bits=tile_bits, low_bits=low_bits, fwd_max_mats=1 << 30)
        # lowering and planning run off the caller's thread, several at once
        # (the C planner releases the interpreter lock)
        self._planner = cf.ThreadPoolExecutor(max_workers=max(1, int(planning_threads)))
        self._planning: dict = {}  # structure key -> Future of its Program
        self.programs: dict = {}
        # compiling runs on one thread (NVRTC already compiles a program's
        # passes in parallel), largest work first; a structure is compiled at
        # most once
        self.compile_min_tiles = None if not compile_min_tiles else int(compile_min_tiles)
        self._compileq = _CompileQueue()
        self._ready: set = set()  # programs whose compiled kernels are loaded (ids)
        self.compile_errors: list = []
        self._plock = threading.Lock()
        self._compiler = threading.Thread(target=self._compile_loop, daemon=True)
        self._compiler.start()
        self.stream = torch.cuda.Stream(device=self.device)
        self._queue = []
        self._cv = threading.Condition()
        self._stop = False
        self._completing = collections.deque()
        self._used = 0
        self.steps = 0
        self.launches = 0
        self.compiled_launches = 0
        self._worker = threading.Thread(target=self._run, daemon=True)
        self._poller = threading.Thread(target=self._poll, daemon=True)
        self._worker.start()
        self._poller.start()

    # -- public --
    def submit(self, desc: dict, arrival: float | None = None) -> Request:
        """Queue one request; returns at once.  Its lowering and planning run
        on the planning threads; a request that cannot be served (a gate the
        loop does not take, more memory than the whole budget) fails its
        future instead of entering the queue."""
        req = Request(desc, arrival)
        self._planner.submit(self._plan, req)
        return req

    def prepare(self, desc: dict) -> Program:
        """Plan a request structure now and, unless compiling is off,
        compile its passes (blocking): a deployment warms the server with its
        circuits before traffic arrives.  Later requests of the structure
        skip planning, and those of at least compile_min_tiles tiles per pass
        run on the compiled kernels."""
        lo = lower_description(desc)[0]
        prog = self._program(lo)
        if self.compile_min_tiles is not None:
            self._compileq.claim(prog)
            with torch.cuda.device(self.device):
                prog.ensure_compiled(self.device)
            with self._plock:
                self._ready.add(id(prog))
        return prog

    @property
    def compiled_programs(self) -> int:
        """Programs whose compiled kernels are loaded."""
        return len(self._ready)

    def _plan(self, req: "Request") -> None:
        try:
            req.lowered = lower_description(req.desc)
            req.prog = self._program(req.lowered[0])
            need = req.need = self._device_bytes(req)
            lo = req.lowered[0]
            tiles = _tiles_per_pass(lo.n, req.desc["batch"] or 1, self.tile_bits)
            req.work = tiles * req.prog.info.forward_passes
        except (ValueError, RuntimeError) as e:
            req.future.set_exception(e)
            return
        if self.compile_min_tiles is not None and tiles >= self.compile_min_tiles and need <= self.budget:
            self._compileq.push(req.prog, req.work)
        if need > self.budget:
            req.future.set_exception(MemoryError(
                f"request needs {need} bytes of device memory (state, workspace, output), more than the "
                f"HBM budget {self.budget}"))
            return
        with self._cv:
            self._queue.append(req)
            self._cv.notify()

    def close(self):
        self._planner.shutdown(wait=True)  # every submitted request is queued or failed
        with self._cv:
            self._stop = True
            self._cv.notify()
        self._worker.join()
        self._poller.join()
        self._compileq.close()  # a compile in progress finishes; queued ones are dropped
        self._compiler.join()

    def _compile_loop(self):
        while True:
            prog = self._compileq.pop()
            if prog is None:
                return
            try:
                with torch.cuda.device(self.device):
                    prog.ensure_compiled(self.device, background=True)
                with self._plock:
                    self._ready.add(id(prog))
            except RuntimeError as e:  # NVRTC missing or failing: the interpreter serves it
                self.compile_errors.append(str(e).splitlines()[0])

    # -- internals --
    @staticmethod
    def _device_bytes(req: "Request") -> int:
        """Device bytes a request holds while admitted: state, workspace
        (each rounded up like the caching allocator's 512-byte blocks) and
        output."""
        lo = req.lowered[0]
        B = req.desc["batch"] or 1
        rnd = lambda x: (int(x) + 511) // 512 * 512  # noqa: E731
        ws = _lib.load().qg_program_workspace_bytes(req.prog.handle, B, 0)
        return rnd((1 << lo.n) * 8 * B) + rnd(max(int(ws), 256)) + rnd(B * lo.n * 4) + rnd(32) * 3

    def _program(self, lo: Lowered) -> Program:
        """The planned program of a structure, planned once: a thread that
        finds another one planning the same structure waits for it."""
        key = structure_key(lo)
        with self._plock:
            p = self.programs.get(key)
            if p is not None:
                return p
            fut = self._planning.get(key)
            mine = fut is None
            if mine:
                fut = self._planning[key] = cf.Future()
        if not mine:
            return fut.result()
        try:
            p = Program(lo, lo.measure, keep_state=False, **self.opts)
        except BaseException as e:
            with self._plock:
                del self._planning[key]
            fut.set_exception(e)
            raise
        with self._plock:
            self.programs[key] = p
            del self._planning[key]
        fut.set_result(p)
        return p

    def _admit(self, req: Request) -> _Slot:
        lo, params, named, shift = req.lowered
        prog = req.prog
        B = req.desc["batch"] or 1
        n = lo.n
        s = _Slot()
        s.req, s.prog, s.batch, s.next_pass, s.shift = req, prog, B, 0, shift
        s.bytes = req.need
        s.tiles = _tiles_per_pass(n, B, self.tile_bits)
        s.idle = 0
        s.compiled = False  # set at the first step after its program's kernels are ready
        dev = self.device
        s.state = torch.empty(B, 1 << n, dtype=torch.complex64, device=dev)
        s.ws = prog.workspace(B, False, dev)
        s.out = torch.empty(B, n, dtype=torch.float32, device=dev)
        s.host_out = torch.empty(B, n, dtype=torch.float32, pin_memory=True)
        s.params = torch.from_numpy(params).pin_memory().to(dev, non_blocking=True)
        s.named = torch.from_numpy(np.ascontiguousarray(named)).pin_memory().to(dev, non_blocking=True)
        s.umats = torch.zeros(1, 2, 2, dtype=torch.complex64, device=dev)
        _lib.call("qg_program_prepare", prog.handle, prog.table(dev).data_ptr(), s.ws.data_ptr(), s.ws.numel(),
                  B, s.params.data_ptr(), s.named.data_ptr(), s.umats.data_ptr(), self.stream.cuda_stream)
        req.admitted = time.perf_counter()
        return s

    def _run(self):
        lib = _lib.load()
        active: list[_Slot] = []
        # events of the steps enqueued and not yet finished: at most
        # max_inflight_steps, so that admission and step selection decide
        # close to when the GPU runs the work (a request that arrives now can
        # go ahead of the remaining passes of larger ones)
        inflight = collections.deque()
        with torch.cuda.device(self.device), torch.cuda.stream(self.stream):
            while True:
                with self._cv:
                    while not self._queue and not active and not self._stop:
                        self._cv.wait()
                    if self._stop and not self._queue and not active:
                        break
                    while self._queue and len(active) < self.max_active:
                        req = self._next_admission()
                        if req is None:
                            break
                        self._queue.remove(req)
                        self._used += req.need
                        active.append(self._admit(req))
                if not active:
                    continue
                while len(inflight) >= self.max_inflight_steps:
                    ev = inflight[0]
                    if ev.query():
                        inflight.popleft()
                    else:
                        time.sleep(20e-6)
                step = self._step_selection(active)
                if self._ready:
                    for s in step:
                        if not s.compiled and id(s.prog) in self._ready and s.tiles >= self.compile_min_tiles:
                            s.compiled = True
                interp = [s for s in step if not s.compiled]
                for base in range(0, len(interp), _lib.MAX_JOBS):
                    chunk = interp[base:base + _lib.MAX_JOBS]
                    jobs = (_lib.Job * len(chunk))()
                    for i, s in enumerate(chunk):
                        jobs[i] = self._job(s)
                    _lib.check(lib.qg_jobs_run_pass(jobs, len(chunk), self.stream.cuda_stream))
                    self.launches += 1
                for s in step:
                    if s.compiled:
                        job = self._job(s)
                        _lib.check(lib.qg_job_run_pass_compiled(ctypes.byref(job), self.stream.cuda_stream))
                        self.launches += 1
                        self.compiled_launches += 1
                self.steps += 1
                ev = torch.cuda.Event()
                ev.record(self.stream)
                inflight.append(ev)
                stepped = set(id(s) for s in step)
                still = []
                for s in active:
                    if id(s) not in stepped:
                        s.idle += 1
                        still.append(s)
                        continue
                    s.idle = 0
                    s.next_pass += 1
                    if s.next_pass < s.prog.info.forward_passes:
                        still.append(s)
                        continue
                    _lib.call("qg_program_finish", s.prog.handle, s.prog.table(self.device).data_ptr(),
                              s.ws.data_ptr(), s.ws.numel(), s.batch, s.out.data_ptr(), self.stream.cuda_stream)
                    s.host_out.copy_(s.out, non_blocking=True)
                    s.event = torch.cuda.Event()
                    s.event.record(self.stream)
                    # stream order makes the memory reusable by later work on this stream
                    with self._cv:
                        self._used -= s.bytes
                        self._completing.append(s)
                active = still

    def _job(self, s: _Slot) -> "_lib.Job":
        # a program without an embedding starts from |0..0> in its first pass
        zero = 1 if (s.next_pass == 0 and not s.prog.info.has_embedding) else 0
        return _lib.Job(s.prog.handle, s.prog.table(self.device).data_ptr(), s.ws.data_ptr(), s.ws.numel(),
                        s.state.data_ptr(), s.batch, s.next_pass, zero, s.out.data_ptr())

    def _next_admission(self):
        """The queued request to admit next, or None when it does not fit the
        budget now (called with the queue lock held)."""
        if self.policy == "all":
            req = min(self._queue, key=lambda r: r.arrival)
            return req if self._used + req.need <= self.budget else None
        now = time.perf_counter()
        oldest = min(self._queue, key=lambda r: r.arrival)  # planning may queue out of arrival order
        if now - oldest.arrival > self.max_queue_wait_s:
            # waited too long: it goes first, and nothing passes it
            return oldest if self._used + oldest.need <= self.budget else None
        fits = [r for r in self._queue if self._used + r.need <= self.budget]
        return min(fits, key=lambda r: r.work) if fits else None

    def _step_selection(self, active):
        """Active requests whose next pass runs in this step."""
        if self.policy == "all":
            return list(active)
        order = sorted(active, key=lambda s: s.remaining())
        step, tiles = [], 0
        for s in order:
            if step and tiles + s.tiles > self.step_tiles and s.idle < self.max_idle_steps:
                continue
            step.append(s)
            tiles += s.tiles
        return step

    def _poll(self):
        while True:
            with self._cv:
                done = self._stop and not self._queue and not self._completing and not self._worker.is_alive()
            if done:
                break
            if not self._completing:
                time.sleep(20e-6)
                continue
            s = self._completing[0]
            if s.event.query():
                self._completing.popleft()
                s.req.completed = time.perf_counter()
                out = s.host_out[:, s.shift:].clone()
                s.req.future.set_result(out)
            else:
                time.sleep(20e-6)


def run_plain(desc: dict, device) -> torch.Tensor:
    """One request through the plain per-gate form (one launch per gate): the
    serving baseline without batching."""
    from . import workloads

    circ = workloads.build_circuit(desc, engine="plain").to(device)
    kw = workloads.circuit_inputs(desc, device)
    with torch.no_grad():
        return circ(**kw)

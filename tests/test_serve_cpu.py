"""Serving-loop host logic on the CPU: QASM requests lower like the
description they were exported from, and a request's HBM need counts its
state, program workspace and output (no GPU needed: planning is host-only)."""
import numpy as np

from qandle_gb300 import _lib, serve, workloads
from qandle_gb300.engine import Program


def test_request_need_counts_state_workspace_and_output():
    rng = np.random.default_rng(5)
    desc = workloads.random_sel_request(rng, n_range=(12, 12), depth_range=(3, 3), batch_max=32)
    req = serve.Request(desc)
    req.lowered = serve.lower_description(desc)
    lo = req.lowered[0]
    req.prog = Program(lo, lo.measure, keep_state=False)
    need = serve.Server._device_bytes(req)
    B = desc["batch"]
    ws = _lib.load().qg_program_workspace_bytes(req.prog.handle, B, 0)
    assert ws > 0
    assert need >= (1 << 12) * 8 * B + ws + B * 12 * 4


def test_qasm_request_lowers_like_its_description():
    desc = workloads.sel_reupload(n=7, batch=3, layers=2, reupload_every=1)
    text = workloads.build_circuit(desc).to_openqasm3()
    x = desc["inputs"]["x"]
    inputs = {}
    for line in text.splitlines():
        if line.startswith("input float "):
            name = line[len("input float "):-1]
            col = int(name[2:]) if name.startswith("up") else int(name.rsplit("_", 1)[1])
            inputs[name] = x[:, col]
    req = serve.description_from_qasm(text, inputs, batch=3)
    lo_q, params_q, named_q, _ = serve.lower_description(req)
    assert lo_q.n == 7 and lo_q.measure == "z"
    # rotations, CNOTs and angle values in the exported order
    from oracle import oracle

    assert np.abs(oracle.forward(req) - oracle.forward(desc)).max() < 1e-12


class _Req:
    def __init__(self, work, need, arrival):
        self.work, self.need, self.arrival = work, need, arrival


class _Prog:
    class info:
        forward_passes = 10


class _Active:
    def __init__(self, tiles, next_pass, idle=0):
        self.tiles, self.next_pass, self.idle, self.prog = tiles, next_pass, idle, _Prog

    def remaining(self):
        return self.tiles * (self.prog.info.forward_passes - self.next_pass)


def _server(policy="srpt", used=0, budget=100):
    import types

    return types.SimpleNamespace(policy=policy, _used=used, budget=budget, max_queue_wait_s=10.0,
                                 step_tiles=100, max_idle_steps=4, _queue=[])


def test_admission_takes_least_work_that_fits():
    import time

    now = time.perf_counter()
    srv = _server(used=60)
    big, small, too_big = _Req(500, 30, now), _Req(5, 10, now), _Req(1, 50, now)
    srv._queue = [big, too_big, small]
    assert serve.Server._next_admission(srv) is small      # least work among those that fit
    srv._queue = [too_big]
    assert serve.Server._next_admission(srv) is None        # nothing fits the budget now
    old = _Req(900, 30, now - 11.0)
    srv._queue = [old, small]
    assert serve.Server._next_admission(srv) is old         # waited too long: goes first
    srv = _server(policy="all", used=0)
    srv._queue = [big, small]
    assert serve.Server._next_admission(srv) is big        # oldest first


def test_step_takes_least_remaining_work_up_to_the_tile_budget():
    srv = _server()
    a, b, c = _Active(tiles=60, next_pass=9), _Active(tiles=30, next_pass=0), _Active(tiles=500, next_pass=5)
    step = serve.Server._step_selection(srv, [c, b, a])
    assert step == [a, b]                                   # remaining 60, 300; c (2500) over the budget
    c.idle = 4
    assert c in serve.Server._step_selection(srv, [c, b, a])  # left out too long: taken
    lone = _Active(tiles=1000, next_pass=0)
    assert serve.Server._step_selection(srv, [lone]) == [lone]  # at least one request per step
    srv = _server(policy="all")
    assert serve.Server._step_selection(srv, [c, b, a]) == [c, b, a]


def test_tiles_per_pass():
    assert serve._tiles_per_pass(20, 3, 13) == 3 << 7
    assert serve._tiles_per_pass(8, 33, 13) == 2             # 32 samples of 2^8 per 2^13 tile
    assert serve._tiles_per_pass(13, 1, 13) == 1


def test_compile_queue_orders_by_work_and_dedupes():
    """The background compile queue hands out programs largest work first,
    takes each program once (also one compiled by prepare), and after close
    hands out nothing."""
    import threading

    q = serve._CompileQueue()
    a, b, c, d = object(), object(), object(), object()
    assert q.push(a, 5) and q.push(b, 50) and q.push(c, 20)
    assert not q.push(b, 500)  # already queued
    q.claim(d)
    assert not q.push(d, 1000)  # compiled elsewhere
    assert [q.pop(), q.pop(), q.pop()] == [b, c, a]
    got = []
    t = threading.Thread(target=lambda: got.append(q.pop()))
    t.start()  # waits for work
    q.close()
    t.join(timeout=10)
    assert not t.is_alive() and got == [None]
    assert not q.push(object(), 1)

"""Bank-conflict freedom of the exchanges, checked on the host.

An exchange writes and reads the tile through a swizzled planar layout in
shared memory: local index j goes to slot j ^ L(j >> 5), L taking the bank
images of the high bits (qandle_gb300/csrc/engine.h, swz_image).  A warp's
access is conflict-free when its five lane bits have linearly independent
bank images over GF(2).  These tests read the image table from the header,
check that it leaves such a lane choice for almost every register set, that
the planner's exchanges on the benchmark circuits all pick one, and that no
lane-dependent pending X (folded into the write addresses) makes an
exchange's writes conflict."""
import itertools
import os
import re

import numpy as np
import pytest

from qandle_gb300 import engine, workloads

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "qandle_gb300", "csrc",
                      "engine.h")


def _images():
    src = open(HEADER).read()
    body = src[src.index("constexpr int swz_image(int k)"):]
    body = body[:body.index(";")]
    vals = [int(v) for v in re.findall(r"\?\s*(\d+)\s*:", body)] + [int(re.findall(r":\s*(\d+)\s*$", body)[0])]
    assert len(vals) == 8
    return [1 << b for b in range(5)] + vals


def _rank(vs):
    basis = []
    for v in vs:
        for e in basis:
            v = min(v, v ^ e)
        if v:
            basis.append(v)
    return len(basis)


@pytest.mark.parametrize("tb,rb,limit", [(13, 5, 3), (12, 4, 1), (13, 4, 0)])
def test_almost_every_register_set_leaves_conflict_free_lanes(tb, rb, limit):
    img = _images()
    bad = sum(1 for regs in itertools.combinations(range(tb), rb)
              if _rank([img[b] for b in range(tb) if b not in regs]) < 5)
    assert bad <= limit


def _lanes(z):
    return [(z >> (4 * k)) & 15 for k in range(5)]


@pytest.mark.parametrize("name", ["sel_reupload", "deep_u", "adjoint_brick"])
def test_planned_exchanges_use_independent_lanes(name):
    desc = getattr(workloads, name)()
    if name == "deep_u":
        desc = workloads.deep_u(n=20, layers=10)
    lo = engine.lower(workloads.build_circuit(desc).circuit)
    img = _images()
    for training in (False, True):
        prog = engine.Program(lo, "probs", keep_state=training, segments=2 if training else 1)
        for backward in ((False, True) if training else (False,)):
            for pd in prog.passes(backward):
                maps = [op for op in pd["ops"] if op[0] == 1]
                for op in maps:
                    assert _rank([img[b] for b in _lanes(op[2])]) == 5, (name, backward)


def _write_map_ranks(pd, rb, tb, img):
    """Rank of each exchange's write lane -> bank map of a planned pass, with
    the pending X of every register tracked through the ops as the global
    bits it depends on (a CNOT controlled by a thread bit makes the target's
    pending X depend on that bit; the exchange folds the pending X into its
    write addresses)."""
    OP_MAP, OP_CX, OP_CZ, OP_SWAP, OP_XMAT, LOC_REG = 1, 4, 5, 6, 8, 0x100
    gbit = pd["gbit"]
    if pd["init"] == 2:
        y, z = pd["init_map"][0], pd["init_map"][1]
    else:
        y = sum((5 + k) << (4 * k) for k in range(rb))
        z = 0x43210
    reg = [(y >> (4 * k)) & 15 for k in range(rb)]
    lane = _lanes(z)
    form = [0] * rb
    ranks = []
    for op in pd["ops"]:
        k, oy, oz, ow = (int(v) for v in op)
        if k == OP_MAP:
            vs = []
            for j in range(5):
                v = img[lane[j]]
                if lane[j] < len(gbit):
                    for r in range(rb):
                        if (form[r] >> gbit[lane[j]]) & 1:
                            v ^= img[reg[r]]
                vs.append(v)
            ranks.append(_rank(vs))
            reg = [(oy >> (4 * q)) & 15 for q in range(rb)]
            lane = _lanes(oz)
            form = [0] * rb
        elif k == OP_CX:
            form[oy] ^= form[oz & 7] if oz & LOC_REG else (1 << oz)
        elif k == OP_SWAP and oy != oz:
            form[oy], form[oz] = form[oz], form[oy]
        elif k == OP_CZ:
            for loc in (oy, oz):
                if loc & LOC_REG:
                    form[loc & 7] = 0
        elif k == OP_XMAT:
            form[oy] = 0
    return ranks


@pytest.mark.parametrize("name", ["sel_reupload", "adjoint_brick", "deep_u"])
def test_exchange_writes_stay_conflict_free_under_pending_x(name):
    """The planner applies a lane-dependent pending X (OP_XMAT) before an
    exchange whose write map it would make singular: every exchange of the
    benchmark circuits, forward and backward, writes without bank
    conflicts, and the headline forward needs OP_XMAT at all."""
    desc = getattr(workloads, name)()
    if name == "deep_u":
        desc = workloads.deep_u(n=20, layers=10)
    lo = engine.lower(workloads.build_circuit(desc).circuit)
    img = _images()
    prog = engine.Program(lo, "p0", keep_state=True, segments=2)
    xmats = 0
    for backward, rb, tb in ((False, 5, 13), (True, 4, 12)):
        for pd in prog.passes(backward):
            assert all(r == 5 for r in _write_map_ranks(pd, rb, tb, img)), (name, backward)
            xmats += int(sum(1 for op in pd["ops"] if op[0] == 8))
    if name == "sel_reupload":
        assert xmats > 0


@pytest.mark.parametrize("seed", range(8))
def test_random_circuit_exchange_writes_conflict_free(seed):
    """Random circuits dense in CNOTs and CZs (many lane-controlled CNOTs,
    hence lane-dependent pending X): every exchange write of their forward
    and backward plans is conflict-free."""
    rng = np.random.default_rng(100 + seed)
    n = 16
    gates = []
    for _ in range(240):
        r = rng.random()
        if r < 0.5:
            gates.append((("rx", "ry", "rz")[rng.integers(3)], int(rng.integers(n)), float(rng.uniform(-3, 3)), None))
        else:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            gates.append(("cnot", a, b) if r < 0.85 else ("cz", a, b))
    desc = {"name": "mix", "n": n, "batch": 2, "gates": gates, "inputs": {}, "measure": "p0", "targets": None}
    lo = engine.lower(workloads.build_circuit(desc).circuit)
    img = _images()
    prog = engine.Program(lo, "p0", keep_state=True, segments=2)
    for backward, rb, tb in ((False, 5, 13), (True, 4, 12)):
        for pd in prog.passes(backward):
            assert all(r == 5 for r in _write_map_ranks(pd, rb, tb, img)), (seed, backward)

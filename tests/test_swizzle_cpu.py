"""Bank-conflict freedom of the exchanges, checked on the host.

An exchange writes and reads the tile through a swizzled planar layout in
shared memory: local index j goes to slot j ^ L(j >> 5), L taking the bank
images of the high bits (qandle_gb300/csrc/engine.h, swz_image).  A warp's
access is conflict-free when its five lane bits have linearly independent
bank images over GF(2).  These tests read the image table from the header,
check that it leaves such a lane choice for almost every register set, and
that the planner's exchanges on the benchmark circuits all pick one."""
import itertools
import os
import re

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

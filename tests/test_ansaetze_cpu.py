"""TwoLocal, SpecialUnitary (SU) and StronglyEntanglingLayerBudget against
the reference (tests/golden/ansaetze.npz, made by running qandle's ansaetze):
parameter count, decompositions, and the output state for fixed angles on a
seeded input -- including the reference's order of the CNOT chain in the
built TwoLocal / SU (applied last pair first).  States are computed from
the built ansatz's `applied_gates` (what both engines run) with the
complex128 oracle; one case per kind is also lowered, planned and emulated as
the fused engine runs it."""
import json
import os

import numpy as np
import pytest
import torch

import qandle_gb300 as q
from oracle import oracle
from tests.golden import make_golden as mg

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = np.load(os.path.join(HERE, "golden", "ansaetze.npz"))
CASES = mg.ansatz_circuits()


def _built(name):
    kind, n, args = CASES[name]
    circ = mg.build_ansatz(q, kind, n, args)
    rec = json.loads(str(GOLDEN[name]))
    with torch.no_grad():
        for p, v in zip(circ.parameters(), rec["params"]):
            p.fill_(v)
    return circ, rec, n


def _desc(mods, n):
    gates = []
    for m in mods:
        kind = type(m).__name__.replace("Built", "").lower()
        if kind in ("cnot", "cz"):
            gates.append((kind, int(m.c), int(m.t)))
        else:  # the fixtures use the identity remapping
            gates.append((kind, int(m.qubit), float(m.theta.detach().reshape(-1)[0]), None))
    return {"n": n, "batch": 1, "gates": gates, "inputs": {}, "measure": "state", "targets": None}


def _psi(n):
    rng = np.random.default_rng(11)
    psi = rng.normal(size=(1 << n,)) + 1j * rng.normal(size=(1 << n,))
    return psi / np.linalg.norm(psi)


@pytest.mark.parametrize("name", sorted(CASES))
def test_structure_matches_reference(name):
    circ, rec, n = _built(name)
    built = circ.circuit.layers[0]
    assert len(list(circ.parameters())) == len(rec["params"])
    assert mg.gate_record(built.decompose()) == rec["built_decompose"]
    if "unbuilt_decompose" in rec:
        kind, _, args = CASES[name]
        assert mg.gate_record(mg.build_unbuilt_ansatz(q, kind, args).decompose()) == rec["unbuilt_decompose"]


@pytest.mark.parametrize("name", sorted(CASES))
def test_state_matches_reference(name):
    circ, rec, n = _built(name)
    got = oracle.run(_desc(circ.circuit.layers[0].applied_gates, n), state=_psi(n))[0]
    ref = np.asarray(GOLDEN[name + "_state"]).reshape(-1)
    assert np.abs(got - ref).max() < 2e-6


@pytest.mark.parametrize("name", ["twolocal_6", "su_6", "budget_6", "budget_sub"])
def test_fused_plan_matches_reference(name):  # (the fused engine takes n >= 5)
    from qandle_gb300 import engine
    from tests import program_emulator as emu
    from tests.test_planner import _runtime

    circ, rec, n = _built(name)
    for m in circ.circuit.layers[0].applied_gates:
        if hasattr(m, "remapping"):
            m.remapping = q.remap.none
    lo = engine.lower(circ.circuit)
    prog = engine.Program(lo, "state", keep_state=False, tile_bits=13, low_bits=6)
    params, named, umats, embed = _runtime(lo, {"n": n, "batch": 1, "inputs": {}}, 1)
    st, _ = emu.run_forward(prog, n, 1, params, named, umats, state=_psi(n).reshape(1, -1), embed=embed)
    assert np.abs(st[0] - np.asarray(GOLDEN[name + "_state"]).reshape(-1)).max() < 2e-6


def test_twins_follow_module_moves():
    circ, _, _ = _built("su_full")
    built = circ.circuit.layers[0]
    circ = circ.double()
    thetas = {id(p) for p in circ.parameters()}
    for m in built.applied_gates:
        if hasattr(m, "theta"):
            assert id(m.theta) in thetas and m.theta.dtype == torch.float64


def test_unbuilt_without_qubits_cannot_decompose():
    with pytest.raises(ValueError):
        q.TwoLocal(depth=1).decompose()
    with pytest.raises(ValueError):
        q.SU(reps=1).decompose()
    with pytest.raises(AssertionError):
        q.StronglyEntanglingLayerBudget(num_qubits_total=3, control_gate=q.SWAP)

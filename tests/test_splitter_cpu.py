"""Circuit splitter on the CPU (qandle_gb300.splitter, mirrors
qandle/splitter/main.py and grouping.py).

* Structure: for every circuit of tests/golden/make_golden.py:split_circuits,
  Circuit.split(k) / Circuit(..., split_max_qubits=k) gives exactly the
  subcircuits (qubit mapping, gates, angles, names) that the reference's own
  splitter gave (tests/golden/splitter.npz).
* Semantics: the gates of the split circuit, in subcircuit order on the
  parent qubits (what the engines run), give the state the reference's split
  circuit gave (complex128 oracle against the fixture), and the unsplit
  circuit's state wherever the reference's grouping keeps the gate order.
* The reference's assertions (one qubit, no CNOT, a qubit without CNOT,
  max_qubits < 2).
"""
import json
import os
import warnings

import numpy as np
import pytest
import torch

import qandle_gb300 as q
from oracle import oracle
from tests.golden import make_golden as mg

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = np.load(os.path.join(HERE, "golden", "splitter.npz"))
CASES = mg.split_circuits()


@pytest.mark.parametrize("name", sorted(CASES))
def test_split_matches_reference_structure(name):
    gates, n, k, via = CASES[name]
    circ = mg.build_split(q, gates, n, k, via)
    assert isinstance(circ.circuit, q.qcircuit.SplittedCircuit)
    assert mg.split_record(circ) == json.loads(str(GOLDEN[name]))


def _desc_of(layers, n, named):
    """Oracle description of gates on the parent qubits; rotation angles
    without remapping (the fixtures' states use the identity)."""
    gates = []
    for la in layers:
        kind = type(la).__name__.replace("Built", "").lower()
        if kind == "cnot":
            gates.append(("cnot", int(la.c), int(la.t)))
        elif la.named:
            gates.append((kind, int(la.qubit), None, la.name))
        else:
            gates.append((kind, int(la.qubit), float(la.theta.detach().reshape(-1)[0]), None))
    inputs = {nm: np.array([v], dtype=np.float32) for nm, v in named.items()}
    return {"n": n, "batch": 1, "gates": gates, "inputs": inputs, "measure": "state", "targets": None}


@pytest.mark.parametrize("name", sorted(CASES))
def test_split_state_matches_reference(name):
    """The split circuit's gates, in subcircuit order on the parent qubits
    (what the engines run), map the fixture's input state to the state the
    reference's split circuit produced.  For three of the random circuits the
    reference's grouping reorders gates that do not commute, so its split
    circuit differs from the unsplit one; the engine reproduces that too."""
    gates, n, k, via = CASES[name]
    split = mg.build_split(q, gates, n, k, via)
    psi, named = mg.split_inputs(n, gates)
    got = oracle.run(_desc_of(split.circuit.layers, n, named), state=psi)[0]
    ref = np.asarray(GOLDEN[name + "_state"]).reshape(-1)
    assert np.abs(got - ref).max() < 2e-6


def test_split_of_order_preserving_circuits_equals_unsplit():
    for name in ("cnot10_k3", "cnot10_k5", "dummy_k2", "sel6_k3", "sel6_k4"):
        gates, n, k, via = CASES[name]
        split = mg.build_split(q, gates, n, k, via)
        whole = q.Circuit(mg.split_layers(q, gates), num_qubits=n)
        psi, named = mg.split_inputs(n, gates)
        a = oracle.run(_desc_of(split.circuit.layers, n, named), state=psi)
        b = oracle.run(_desc_of(whole.circuit.layers, n, named), state=psi)
        assert np.abs(a - b).max() < 1e-10, name


def test_split_shares_parameters_with_subcircuits():
    gates, n, k, via = CASES["sel6_k3"]
    split = mg.build_split(q, gates, n, k, via)
    sub = [p for sc in split.circuit.subcircuits for p in sc.parameters()]
    twins = [la.theta for la in split.circuit.layers if hasattr(la, "theta")]
    assert len(sub) == len(twins) == 36
    assert {id(p) for p in sub} == {id(p) for p in twins}
    assert len(list(split.parameters())) == 36


def test_split_again_warns_and_returns_itself():
    gates, n, k, via = CASES["cnot10_k5"]
    split = mg.build_split(q, gates, n, k, via)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        assert split.split(max_qubits=3) is split
    assert any("already split" in str(x.message) for x in w)


def test_split_qasm_maps_qubits_back():
    gates, n, k, via = CASES["cnot10_k5"]
    split = mg.build_split(q, gates, n, k, via)
    whole = q.Circuit(mg.split_layers(q, gates), num_qubits=n)
    assert split.to_openqasm2().splitlines()[4:] == whole.to_openqasm2().splitlines()[4:]
    with pytest.raises(NotImplementedError):
        split.to_matrix()


def test_reference_assertions():
    with pytest.raises(AssertionError):
        q.Circuit([q.CNOT(0, 1), q.RX(2, theta=0.1)], num_qubits=3).split(max_qubits=2)  # qubit 2 has no CNOT
    with pytest.raises(AssertionError):
        q.Circuit([q.RX(0, theta=0.1), q.RY(1, theta=0.2)], num_qubits=2).split(max_qubits=2)  # no CNOT
    with pytest.raises(AssertionError):
        q.Circuit([q.CNOT(0, 1), q.CNOT(1, 2)], num_qubits=3).split(max_qubits=1)
    with warnings.catch_warnings(record=True):
        warnings.simplefilter("always")
        one = q.qcircuit.UnsplittedCircuit(1, [q.RX(0, theta=0.1)])
        assert one.split(max_qubits=2) is one


def test_unsplit_when_small_enough():
    c = q.Circuit([q.CNOT(0, 1), q.CNOT(1, 2)], num_qubits=3, split_max_qubits=3)
    assert not isinstance(c.circuit, q.qcircuit.SplittedCircuit)
    assert torch.is_tensor(c.circuit.state)


@pytest.mark.parametrize("name", ["cnot10_k5", "sel6_k3", "random1_k3", "random2_k3"])
def test_fused_plan_of_split_circuit_matches_reference(name):
    """The fused engine lowers a split circuit from its `layers` (the
    subcircuits' gates on the parent qubits); the planned program, run by the
    op emulator, gives the reference's split state."""
    from qandle_gb300 import engine
    from tests import program_emulator as emu
    from tests.test_planner import _runtime

    gates, n, k, via = CASES[name]
    split = mg.build_split(q, gates, n, k, via)
    for la in split.circuit.layers:  # the fixture's states use no remapping
        if hasattr(la, "remapping"):
            la.remapping = q.remap.none
    lo = engine.lower(split.circuit)
    prog = engine.Program(lo, "state", keep_state=False, tile_bits=13, low_bits=6)
    psi, named = mg.split_inputs(n, gates)
    desc = {"n": n, "batch": 1, "inputs": {nm: np.array([v], np.float32) for nm, v in named.items()}}
    params, named_t, umats, embed = _runtime(lo, desc, 1)
    st, _ = emu.run_forward(prog, n, 1, params, named_t, umats, state=psi.reshape(1, -1), embed=embed)
    assert np.abs(st[0] - np.asarray(GOLDEN[name + "_state"]).reshape(-1)).max() < 2e-6


def test_module_moves_reach_the_twins():
    """Module.to / .cuda() reach the twins (not registered as submodules):
    their thetas stay the subcircuits' Parameters and their buffers move."""
    gates, n, k, via = CASES["dummy_k2"]
    layers = mg.split_layers(q, gates) + [q.U(1, matrix=torch.eye(2, dtype=torch.complex64)), q.CNOT(1, 0)]
    split = q.Circuit(layers, num_qubits=n).split(max_qubits=2)
    split = split.double()
    seen_u = False
    for sc in split.circuit.subcircuits:
        for la, tw in zip(sc.layers, sc.twins):
            if hasattr(la, "theta"):
                assert tw.theta is la.theta and la.theta.dtype == torch.float64
            if hasattr(tw, "_m"):
                seen_u = True
                assert tw._m.dtype == la._m.dtype
    assert seen_u


def test_deepcopy_keeps_twins_on_the_copied_parameters():
    import copy

    gates, n, k, via = CASES["sel6_k3"]
    d = copy.deepcopy(mg.build_split(q, gates, n, k, via))
    params = {id(p) for p in d.parameters()}
    twins = [la for la in d.circuit.layers if hasattr(la, "theta")]
    assert len(params) == len(twins) == 36
    assert all(id(t.theta) in params for t in twins)

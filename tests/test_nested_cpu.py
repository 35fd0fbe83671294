"""Circuits used as layers of another circuit (qandle allows it: they are
modules).  The fused engine lowers a nested circuit's layers inline: the
lowering equals that of the decomposed circuit, and the planned program,
emulated, equals the oracle."""
import numpy as np
import pytest
import torch

import qandle_gb300 as q
from oracle import oracle
from qandle_gb300 import engine
from tests import program_emulator as emu
from tests.test_planner import _runtime


def _nested(n=6):
    c1 = q.Circuit(layers=[q.RX(0, theta=0.3, remapping=None), q.CNOT(0, 1)], num_qubits=n)
    c2 = q.Circuit(layers=[q.RY(1, theta=-0.8, remapping=None),
                           q.StronglyEntanglingLayer(qubits=list(range(1, n)), remapping=None)], num_qubits=n)
    inner = q.Circuit(layers=[c2, q.CNOT(n - 1, 0)], num_qubits=n)
    return q.Circuit(layers=[c1, q.RZ(0, theta=1.1, remapping=None), inner], num_qubits=n)


def test_nested_lowering_equals_decomposed():
    c = _nested()
    lo, ld = engine.lower(c.circuit), engine.lower(c.decompose().circuit)
    assert lo.gates == ld.gates
    assert [float(m.theta.detach()) for m in lo.param_mods] == [float(m.theta.detach()) for m in ld.param_mods]
    # the nested modules' parameters are the ones the program reads
    ids = {id(p) for p in c.parameters()}
    assert all(id(m.theta) in ids for m in lo.param_mods)


def test_nested_plan_matches_oracle():
    n = 6
    c = _nested(n)
    lo = engine.lower(c.circuit)
    prog = engine.Program(lo, "state", keep_state=False)
    params, named, umats, embed = _runtime(lo, {"n": n, "batch": 1, "inputs": {}}, 1)
    st, _ = emu.run_forward(prog, n, 1, params, named, umats, embed=embed)
    gates = []
    for m in c.decompose().circuit.layers:
        kind = type(m).__name__.replace("Built", "").lower()
        if kind == "cnot":
            gates.append(("cnot", m.c, m.t))
        else:
            gates.append((kind, m.qubit, float(m.remapping(m.theta).detach().reshape(-1)[0]), None))
    ref = oracle.run({"n": n, "batch": 1, "gates": gates, "inputs": {}, "measure": "state", "targets": None})
    assert np.abs(st - ref).max() < 1e-10


def test_nested_width_mismatch_is_refused():
    small = q.Circuit(layers=[q.CNOT(0, 1)], num_qubits=2)
    big = q.Circuit(layers=[small, q.CNOT(2, 3)], num_qubits=6)
    with pytest.raises(ValueError):
        engine.lower(big.circuit)


def test_per_gate_path_flattens_nested_circuits_and_ansaetze():
    """The per-gate in-place path (inference without autograd) runs a nested
    circuit's layers and an ansatz's applied gates in place, in order; the
    flattened list equals the decomposed circuit's gates."""
    from qandle_gb300 import plain

    n = 6
    c = _nested(n)
    flat = plain._flat_layers(list(c.circuit.layers), n)
    dec = list(c.decompose().circuit.layers)
    assert [str(m) for m in flat] == [str(m) for m in dec]
    small = q.Circuit(layers=[q.CNOT(0, 1)], num_qubits=2)
    with pytest.raises(ValueError):
        plain._flat_layers([small], n)


def test_circuit_copies_after_planning():
    """copy.deepcopy, pickling and torch.save of a circuit whose fused
    executor has planned a program leave the executor out (it holds library
    handles); the copy has its own parameters and plans again when called."""
    import copy
    import io
    import pickle

    c = q.Circuit([q.RX(i, theta=0.1 * i, remapping=None) for i in range(6)] + [q.CNOT(0, 1)], num_qubits=6)
    c._executor = engine.FusedExecutor(c.circuit)
    c._executor.program(False)  # planned on the host
    d = copy.deepcopy(c)
    assert d._executor is None and c._executor is not None
    assert [p.detach().item() for p in d.parameters()] == [p.detach().item() for p in c.parameters()]
    assert all(a is not b for a, b in zip(d.parameters(), c.parameters()))
    e = pickle.loads(pickle.dumps(c))
    assert e._executor is None and len(list(e.parameters())) == 6
    buf = io.BytesIO()
    torch.save(c, buf)


def test_decompose_and_split_keep_engine_options():
    c = q.Circuit([q.RX(0, theta=0.1, remapping=None), q.CNOT(0, 1), q.CNOT(1, 2)], num_qubits=3,
                  engine="plain", tile_bits=12)
    for d in (c.decompose(), c.split(max_qubits=2)):
        assert d.engine == "plain" and d._engine_options == {"tile_bits": 12}

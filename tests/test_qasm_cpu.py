"""OpenQASM export equals the reference's text for the same circuits (the
random hash in generated embedding / measurement names normalised), and
ingest reads the export back into the same circuit."""
import re

import numpy as np
import pytest

import qandle_gb300 as q
from tests import golden_io


def _norm(text: str) -> str:
    return re.sub(r"_-?\d{5,}_", "_H_", text)


def _circuits():
    # the same constructions as tests/golden/make_golden.py:qasm_circuits
    return {
        "rot_fixed": ([q.RX(0, theta=0.25, remapping=None), q.RY(1, theta=-1.5, remapping=None),
                       q.RZ(2, theta=3.0, remapping=None), q.CNOT(0, 2), q.CZ(1, 2), q.MeasureProbability()], 3),
        "named": ([q.AngleEmbedding(name="x", qubits=[0, 1, 2], rotation="ry"), q.RZ(1, name="up", remapping=None),
                   q.CNOT(2, 0), q.MeasureProbability()], 3),
        "special": ([q.Reset(qubit=1), q.Controlled(0, q.RY(1, theta=0.5, remapping=None)),
                     q.Invert(q.RX(2, theta=0.75, remapping=None).build(num_qubits=3))], 3),
    }


@pytest.mark.parametrize("name", ["rot_fixed", "named", "special"])
def test_export_matches_reference(name):
    z = golden_io.load("qasm")
    layers, n = _circuits()[name]
    circ = q.Circuit(layers, num_qubits=n)
    assert _norm(circ.to_openqasm2()) == _norm(str(z[f"{name}_qasm2"]))
    assert _norm(circ.to_openqasm3()) == _norm(str(z[f"{name}_qasm3"]))


@pytest.mark.parametrize("name", ["rot_fixed", "named"])
def test_ingest_round_trip(name):
    layers, n = _circuits()[name]
    text = q.Circuit(layers, num_qubits=n).to_openqasm2()
    again = q.Circuit.from_qasm(text)
    assert again.num_qubits == n
    # the embedding comes back as its named rotations
    assert _norm(again.to_openqasm2()) == _norm(text)


def test_ingest_rejects_unknown_lines():
    with pytest.raises(ValueError):
        q.qasm.parse("OPENQASM 2.0;\nqreg q[2];\nccx q[0], q[1], q[2];\n")
    layers, n = q.qasm.parse("OPENQASM 2.0;\nqreg q[2];\nrx(pi/2) q[0];\nswap q[0], q[1];\n")
    assert n == 2 and abs(layers[0].theta.item() - np.pi / 2) < 1e-6


def test_serving_request_from_qasm():
    from qandle_gb300 import serve

    text = ("OPENQASM 3.0;\nqubit[6] q;\nbit[6] c;\ninput float x0;\n"
            "rx(x0) q[0];\nry(0.5) q[1];\ncx q[0], q[1];\ncz q[2], q[3];\nswap q[4], q[5];\n"
            "measure q[0] -> c[0];\n")
    d = serve.description_from_qasm(text, {"x0": np.arange(3, dtype=np.float32)}, batch=3)
    assert d["n"] == 6 and d["batch"] == 3
    assert d["gates"] == [("rx", 0, None, "x0"), ("ry", 1, 0.5, None), ("cnot", 0, 1), ("cz", 2, 3),
                          ("swap", 4, 5)]
    lo, params, named, shift = serve.lower_description(d)
    assert named.shape == (3, 1) and shift == 0

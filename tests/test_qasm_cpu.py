"""OpenQASM export equals the reference's text for the same circuits (the
random hash in generated embedding / measurement names normalised), and
ingest reads the export back into the same circuit."""
import re

import numpy as np
import pytest

import qandle_gb300 as q
from tests import golden_io
from tests.golden import make_golden as mg


def _norm(text: str) -> str:
    return re.sub(r"_-?\d{5,}_", "_H_", text)


def _circuit(name):
    """Circuit `name` of tests/golden/make_golden.py:qasm_circuits, built with
    this package while the default remapping is the identity (the built
    TwoLocal's rotations take the default, as when the fixtures were made)."""
    saved = q.config.DEFAULT_MAPPING
    q.config.DEFAULT_MAPPING = q.remap.none
    try:
        layers, n = mg.qasm_circuits(q)[name]
        return q.Circuit(layers, num_qubits=n)
    finally:
        q.config.DEFAULT_MAPPING = saved


@pytest.mark.parametrize("name", ["rot_fixed", "named", "special", "sel", "twolocal", "u_swap", "nested"])
def test_export_matches_reference(name):
    z = golden_io.load("qasm")
    circ = _circuit(name)
    assert _norm(circ.to_openqasm2()) == _norm(str(z[f"{name}_qasm2"]))
    assert _norm(circ.to_openqasm3()) == _norm(str(z[f"{name}_qasm3"]))


@pytest.mark.parametrize("name", ["rot_fixed", "named"])
def test_ingest_round_trip(name):
    circ = _circuit(name)
    n = circ.num_qubits
    text = circ.to_openqasm2()
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

"""Errors and string forms of the front end that user code can observe,
matching the reference's (exception types as qandle raises them, checked by
running qandle on the same calls):

* permutation gates built with a wire >= num_qubits raise ValueError
  (the negative shift count in operators.py:546-555, :580-588, :661-671);
* Reset of a wire outside the circuit raises a RuntimeError (the subsystem
  reshape at operators.py:608-610 raises einops' RuntimeError subclass);
* an unbuilt rotation without angle or name has no OpenQASM form
  (errors.UnbuiltGateError, operators.py:186-203);
* an unbuilt rotation prints the branches of operators.py:177-184 as they
  are (an unnamed gate prints its absent name);
* constructor assertions (operators.py:164-165, :402, :522).
"""
import pytest
import torch

import qandle_gb300 as q


@pytest.mark.parametrize("make", [
    lambda: q.CNOT(5, 0).build(num_qubits=3),
    lambda: q.CNOT(0, 3).build(num_qubits=3),
    lambda: q.CZ(0, 3).build(num_qubits=3),
    lambda: q.CZ(4, 0).build(num_qubits=3),
    lambda: q.SWAP(0, 3).build(num_qubits=3),
    lambda: q.SWAP(4, 0).build(num_qubits=3),
])
def test_out_of_range_wires_raise_value_error(make):
    with pytest.raises(ValueError, match="negative shift count"):
        make()


def test_in_range_wires_build():
    assert isinstance(q.CNOT(0, 2).build(num_qubits=3), q.operators.BuiltCNOT)
    assert isinstance(q.SWAP(1, 1).build(num_qubits=3), q.operators.BuiltSWAP)
    assert isinstance(q.RX(5, theta=0.1).build(num_qubits=3), q.operators.BuiltRX)  # lazy, as in qandle


def test_reset_out_of_range_raises_runtime_error():
    with pytest.raises(RuntimeError):
        q.Reset(3).build(num_qubits=3)
    assert str(q.Reset(2).build(num_qubits=3)) == "Reset 2"


def test_unbuilt_rotation_without_angle_has_no_qasm():
    with pytest.raises(q.errors.UnbuiltGateError):
        q.RX(1).to_qasm()
    assert isinstance(q.errors.UnbuiltGateError("x"), ValueError)
    assert q.RX(1, name="a").to_qasm().qasm3_inputs == "a"


def test_unbuilt_rotation_strings():
    assert str(q.RX(1)) == "RX1 (None)"
    assert str(q.RY(2, theta=0.5)) == "RY2 (None)"
    assert str(q.RZ(0, name="a")) == "RZ0"
    assert str(q.RX(1, theta=0.5, name="a", remapping=None)) == "RX1 (0.50)"
    assert str(q.Controlled(0, q.RX(1, theta=0.5))) == "Controlled 0|RX1 (None)"
    assert str(q.Invert(q.RX(1, theta=0.5))) == "RX1 (None)^-1"


def test_built_strings():
    assert str(q.RX(1, theta=0.5, remapping=None).build(num_qubits=3)) == "RX_1 (0.50)"
    assert str(q.RX(1, name="a").build(num_qubits=3)) == "RX_1 (a)"
    assert str(q.CNOT(0, 2)) == str(q.CNOT(0, 2).build(num_qubits=3)) == "CNOT 0|2"
    assert (str(q.SWAP(0, 2)), str(q.SWAP(0, 2).build(num_qubits=3))) == ("Swap 0|2", "SWAP 0|2")
    assert str(q.U(1, matrix=torch.eye(2)).build(num_qubits=3)) == "U_1"
    assert str(q.Controlled(0, q.RX(1, theta=0.5, remapping=None)).build(num_qubits=3)) == \
        "Controlled 0|RX_1 (0.50)"


def test_constructor_assertions():
    for make in (lambda: q.CNOT(1, 1), lambda: q.CZ(2, 2), lambda: q.RX(-1, theta=0.1),
                 lambda: q.RX(1.0, theta=0.1)):
        with pytest.raises(AssertionError):
            make()


def test_custom_backwards_refuse_double_differentiation():
    """The kernels' backward passes are first-order only; each is marked
    once-differentiable, so create_graph=True followed by a second backward
    raises instead of returning silently wrong higher-order gradients."""
    from qandle_gb300 import engine, plain

    fns = [engine._FusedRun] + [v for v in vars(plain).values()
                                if isinstance(v, type) and issubclass(v, torch.autograd.Function)
                                and v is not torch.autograd.Function]
    assert len(fns) >= 11
    for f in fns:
        assert hasattr(f.backward, "__wrapped__"), f.__name__

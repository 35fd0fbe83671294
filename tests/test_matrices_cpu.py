"""to_matrix(), the inspection half of the operator API, against the
reference (tests/golden/matrices.npz, made by running qandle's to_matrix on
the same modules; tests/golden/make_golden.py:matrix_ops builds them for
either package).

What is pinned: each gate's dense 2^n x 2^n row-form matrix
(operators.py:60-69, :265-305), a named rotation's batch of matrices, Invert
as the matrix inverse (:455-456), Controlled returning its target's matrix
(:514-515), a measurement's identity (measurements.py:55-59), and the
composition of ansaetze (ansaetze/ansatz.py:26-33) and circuits
(qcircuit.py:208-212) by utils.reduce_dot, which multiplies later gates from
the left and adds a batch axis.  Reset and embeddings have no matrix."""
import numpy as np
import pytest
import torch

import qandle_gb300 as q
from tests.golden import make_golden as mg
from tests import golden_io

GOLDEN = golden_io.load("matrices")


def _ours():
    saved = q.config.DEFAULT_MAPPING
    q.config.DEFAULT_MAPPING = q.remap.none
    try:
        return mg.matrix_ops(q)
    finally:
        q.config.DEFAULT_MAPPING = saved


OPS = _ours()


@pytest.mark.parametrize("name", sorted(GOLDEN.files))
def test_to_matrix_matches_reference(name):
    kw = {"a": torch.tensor(mg.MATRIX_NAMED)} if name == "rx_named" else {}
    torch.manual_seed(mg.MATRIX_SEED)
    with torch.no_grad():
        got = OPS[name].to_matrix(**kw)
    ref = GOLDEN[name]
    assert tuple(got.shape) == ref.shape
    assert got.dtype == (torch.float32 if ref.dtype == np.float32 else torch.complex64)
    assert np.abs(got.numpy() - ref).max() < 1e-6


def test_every_fixture_has_a_module():
    assert set(OPS) == set(GOLDEN.files)


def test_no_matrix_for_reset_and_embeddings():
    n = mg.MATRIX_QUBITS
    with pytest.raises(ValueError):
        q.Reset(qubit=1).build(num_qubits=n).to_matrix()
    with pytest.raises(ValueError):
        q.AngleEmbedding(name="x", qubits=[0, 1, 2]).build(num_qubits=n).to_matrix()
    with pytest.raises(NotImplementedError):
        q.Circuit([q.CNOT(0, 1), q.CNOT(1, 2)], num_qubits=3).split(max_qubits=2).to_matrix()


def test_rotation_matrix_is_the_gate_on_a_row_state():
    """For a single gate, state @ to_matrix() is the gate's action: the
    complex128 oracle's RY on a basis row agrees with the matrix row."""
    from oracle import oracle

    n = mg.MATRIX_QUBITS
    mat = OPS["ry_q1"].to_matrix().numpy().astype(np.complex128)
    for i in range(1 << n):
        e = np.zeros((1, 1 << n), np.complex128)
        e[0, i] = 1.0
        out = oracle.run({"n": n, "batch": 1, "gates": [("ry", 1, 0.543321, None)], "inputs": {}}, state=e)
        assert np.abs(out[0] - mat[i]).max() < 1e-6

"""Public helpers mirroring qandle/utils.py: reduce_dot, parse_rot,
do_not_implement, get_matrix_transforms (index mapping checked against an
explicit bit permutation)."""
import numpy as np
import pytest
import torch

import qandle_gb300 as q


def test_reduce_dot_applies_later_matrices_last():
    g = torch.Generator().manual_seed(0)
    a, b, c = (torch.randn(4, 4, generator=g) for _ in range(3))
    batch = torch.randn(3, 4, 4, generator=g)
    assert torch.allclose(q.reduce_dot(a, b, c), (c @ b @ a).unsqueeze(0))
    assert torch.allclose(q.reduce_dot(a, batch), batch @ a)
    assert q.reduce_dot(a) is a
    with pytest.raises(ValueError):
        q.reduce_dot(a, torch.randn(1, 1, 4, 4))


def test_parse_rot():
    assert q.parse_rot("rx") is q.RX and q.parse_rot("RY") is q.RY and q.parse_rot("z") is q.RZ
    with pytest.raises(ValueError):
        q.parse_rot("rw")


def test_do_not_implement():
    meta = q.do_not_implement("forward", reason="no forward here")
    with pytest.raises(AttributeError, match="no forward here"):
        class Bad(metaclass=meta):  # noqa: F841
            def forward(self):
                pass

    class Fine(metaclass=meta):
        def other(self):
            return 1

    assert Fine().other() == 1


@pytest.mark.parametrize("n,qubits", [(5, [1, 3]), (6, [4, 0, 2]), (4, [0, 1, 2, 3]), (7, [6])])
def test_get_matrix_transforms_index_mapping(n, qubits):
    to_matrix, to_state = q.get_matrix_transforms(n, qubits)
    B = 3
    x = torch.arange(B * (1 << n), dtype=torch.float64).reshape(B, 1 << n)
    y = to_matrix(x)
    m = len(qubits)
    outer = [w for w in range(n) if w not in qubits]
    assert y.shape == (B << (n - m), 1 << m)
    for b in range(B):
        for i in range(1 << n):
            bits = [(i >> (n - 1 - w)) & 1 for w in range(n)]  # qubit w is bit n-1-w
            row = b
            for w in outer:
                row = row * 2 + bits[w]
            col = 0
            for w in qubits:
                col = col * 2 + bits[w]
            assert y[row, col] == x[b, i]
    assert torch.equal(to_state(y), x)

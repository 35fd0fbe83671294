"""QConv's argument checks on the CPU (mirrors qandle/test/test_convolution.py
test_errors: a wrong channel count and inputs that are not 4-D raise
ValueError before any work is done)."""
import pytest
import torch

import qandle_gb300 as q


@pytest.mark.parametrize("shape", [(10, 4, 17, 18), (10, 3, 17), (10, 3, 17, 18, 19)])
def test_errors(shape):
    conv = q.QConv(in_channels=3, out_channels=10, kernel_size=3, padding=1)
    with pytest.raises(ValueError):
        conv(torch.rand(*shape))


def test_parameter_layout():
    """A 3x3x3 patch needs ceil(log2 27) = 5 qubits; the parameters are the
    5 x 3 angles of the circuit's one strongly entangling layer
    (convolution.py:27-40)."""
    conv = q.QConv(in_channels=3, out_channels=10, kernel_size=3, padding=1)
    assert conv.qubits == 5
    params = list(conv.parameters())
    assert len(params) == 15 and all(p.dtype == torch.float32 for p in params)

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


def test_patch_layout_and_scaling_equal_the_reference():
    """With the reference's own circuit in place of the engine (CPU, torch),
    QConv's patch gather, shift, channel slice, scale and output layout give
    the reference QConv's output exactly -- also with all-zero patches."""
    import os

    from oracle import reference_torch as rt

    src = "/root/reference/src"
    path = src if os.path.isdir(os.path.join(src, "qandle")) else rt.REF_DIR
    if rt.unavailable_reason(path):
        pytest.skip(rt.unavailable_reason(path))
    qandle = rt.import_reference(path)
    torch.manual_seed(0)
    ref = qandle.QConv(in_channels=2, out_channels=3, kernel_size=3, padding=1)
    for m in ref.qcircuit.circuit.layers[1].mods:
        m.remapping = q.remap.none  # the stand-in has no tanh; parity uses remapping=None
    mine = q.QConv(in_channels=2, out_channels=3, kernel_size=3, padding=1, engine="plain")
    mine.load_state_dict(ref.state_dict(), strict=True)
    mine.qcircuit = ref.qcircuit
    x = torch.rand(2, 2, 5, 6)
    x[:, :, :2, :2] = 0
    with torch.no_grad():
        a, b = mine(x), ref(x)
    assert a.shape == b.shape == (2, 3, 5, 6)
    assert torch.equal(a, b)

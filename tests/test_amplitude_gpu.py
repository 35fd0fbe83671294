"""AmplitudeEmbedding and QConv on the GPU against the reference's golden
outputs (padding and normalisation variants, the input gradient through an
embedded circuit in both engines, two QConv shapes), and an amplitude-
embedded 14-qubit circuit through the fused engine against the oracle."""
import json

import numpy as np
import pytest
import torch

import qandle_gb300 as q
from oracle import oracle
from tests import golden_io

pytestmark = pytest.mark.gpu

TOL = 1e-5


def test_amplitude_embedding_golden(cuda_device):
    z = golden_io.load("amplitude")
    for i in range(int(z["count"])):
        spec = json.loads(str(z[f"a{i}_spec"]))
        n = spec["n"]
        op = q.AmplitudeEmbedding(name="x", qubits=list(range(n)), normalize=spec["normalize"],
                                  pad_with=spec["pad"]).build(num_qubits=n)
        out = op(x=torch.tensor(z[f"a{i}_x"]).to(cuda_device))
        assert np.abs(out.cpu().numpy() - z[f"a{i}_out"]).max() < TOL, spec


@pytest.mark.parametrize("engine", ["plain", "fused"])
def test_amplitude_gradient_vs_reference(cuda_device, engine):
    z = golden_io.load("amplitude")
    n = 3
    th = [float(v) for v in z["grad_th"]]
    layers = [q.AmplitudeEmbedding(name="x", qubits=list(range(n)), normalize=True, pad_with=0.0)]
    layers += [q.RY(qubit=k, theta=th[k], remapping=None) for k in range(n)]
    layers += [q.CNOT(0, 1), q.CNOT(1, 2), q.MeasureProbability()]
    circ = q.Circuit(layers, num_qubits=n, engine=engine).to(cuda_device)
    x = torch.tensor(z["grad_x"], device=cuda_device, requires_grad=True)
    p0 = circ(x=x)
    assert np.abs(p0.detach().cpu().numpy() - z["grad_p0"]).max() < TOL
    (p0 * torch.arange(1, n + 1, device=cuda_device)).sum().backward()
    assert np.abs(x.grad.cpu().numpy() - z["grad_dx"]).max() < 1e-4


@pytest.mark.parametrize("ci", [0, 1])
def test_qconv_golden(cuda_device, ci):
    z = golden_io.load("amplitude")
    cfg = json.loads(str(z[f"qconv{ci}_cfg"]))
    conv = q.QConv(in_channels=cfg["c_in"], out_channels=cfg["c_out"], padding=cfg["padding"])
    thetas = [float(v) for v in z[f"qconv{ci}_thetas"]]
    rots = [m for m in conv.qcircuit.circuit.layers[1].mods if hasattr(m, "theta")]
    assert len(rots) == len(thetas)
    with torch.no_grad():
        for m, t in zip(rots, thetas):
            m.theta.copy_(torch.tensor(t))
            m.remapping = q.remap.none
    conv = conv.to(cuda_device)
    y = conv(torch.tensor(z[f"qconv{ci}_x"]).to(cuda_device))
    ref = z[f"qconv{ci}_out"]
    assert tuple(y.shape) == ref.shape
    assert np.abs(y.detach().cpu().numpy() - ref).max() < TOL


@pytest.mark.parametrize("compiled", [True, False], ids=["compiled", "interpreted"])
def test_amplitude_embedded_circuit_vs_oracle(cuda_device, compiled):
    n, B, L = 14, 3, (1 << 14) - 100
    rng = np.random.default_rng(4)
    x = (rng.random((B, L)) + 0.05).astype(np.float32)
    layers = [q.AmplitudeEmbedding(name="x", qubits=list(range(n)), normalize=True, pad_with=0.5)]
    gates = []
    for w in range(n):
        th = float(np.float32(rng.uniform(0, 6)))
        layers.append(q.RY(qubit=w, theta=th, remapping=None))
        gates.append(("ry", w, th, None))
    for w in range(n - 1):
        layers.append(q.CNOT(w, w + 1))
        gates.append(("cnot", w, w + 1))
    layers.append(q.MeasureProbability())
    circ = q.Circuit(layers, num_qubits=n, compiled=compiled).to(cuda_device)
    p0 = circ(x=torch.tensor(x, device=cuda_device))
    st = np.concatenate([x, np.full((B, 100), 0.5, np.float32)], 1).astype(np.float64)
    st = st / np.linalg.norm(st, axis=1, keepdims=True)
    desc = {"n": n, "batch": B, "gates": gates, "inputs": {}, "measure": "p0"}
    ref = oracle.forward(desc, state=st.astype(np.complex128))
    assert np.abs(p0.detach().cpu().numpy() - ref).max() < TOL

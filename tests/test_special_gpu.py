"""Invert, Controlled and Reset on the GPU: every reference golden case
through the per-layer (plain) and circuit (fused) front ends, the angle
gradient through controlled rotations against the reference's autograd, and
a 14-qubit circuit mixing them through the fused engine (compiled and
interpreted, forward and adjoint) against the complex128 oracle."""
import json
import warnings

import numpy as np
import pytest
import torch

import qandle_gb300 as q
from oracle import oracle
from tests import golden_io

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _cases():
    z = golden_io.load("special")
    return z, int(z["count"])


@pytest.mark.parametrize("engine", ["plain", "fused"])
def test_special_golden(cuda_device, engine):
    z, count = _cases()
    for i in range(count):
        spec = json.loads(str(z[f"s{i}_spec"]))
        n = spec["n"]
        layers = golden_io.special_layers(q, spec, n)
        if spec.get("measure") == "probs":
            layers.append(q.MeasureJointProbability())
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            circ = q.Circuit(layers, num_qubits=n, engine=engine).to(cuda_device)
        inp = torch.tensor(z[f"s{i}_in"]).to(cuda_device)
        kw = {k[len(f"s{i}_kw_"):]: torch.tensor(z[k]).to(cuda_device)
              for k in z.files if k.startswith(f"s{i}_kw_")}
        with torch.no_grad():
            out = circ(inp, **kw)
        ref = z[f"s{i}_out"]
        got = out.detach().cpu().numpy().reshape(ref.shape)
        assert np.abs(got - ref).max() < TOL, (i, spec)


@pytest.mark.parametrize("engine", ["plain", "fused"])
def test_controlled_gradients_vs_reference(cuda_device, engine):
    z, _ = _cases()
    th = [float(v) for v in z["grad_thetas"]]
    layers = [q.RY(qubit=0, theta=th[0], remapping=None), q.CNOT(0, 1),
              q.Controlled(1, q.RX(qubit=2, theta=th[1], remapping=None)),
              q.Controlled(2, q.RY(qubit=3, theta=th[2], remapping=None)),
              q.Controlled(3, q.RZ(qubit=0, theta=th[3], remapping=None)),
              q.MeasureProbability()]
    circ = q.Circuit(layers, num_qubits=4, engine=engine).to(cuda_device)
    inp = torch.tensor(z["grad_in"]).to(cuda_device)
    p0 = circ(inp)
    assert np.abs(p0.detach().cpu().numpy() - z["grad_p0"]).max() < TOL
    (p0 * torch.arange(1, 5, device=cuda_device)).sum().backward()
    params = [m.theta for m in circ.circuit.layers if hasattr(m, "theta")] + \
             [m.t.theta for m in circ.circuit.layers if hasattr(m, "t") and hasattr(m.t, "theta")]
    got = np.array([float(p.grad) for p in params])
    assert np.abs(got - z["grad_out"]).max() < 1e-4


def _mixed(n=14, batch=3, seed=5):
    """A circuit mixing Controlled (fixed and named), Invert and the usual
    gates; returns (front-end layers, oracle description, inputs)."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, np.pi, size=(batch,)).astype(np.float32)
    layers, gates = [], []
    for d in range(3):
        for w in range(n):
            th = float(np.float32(rng.uniform(0, 2 * np.pi)))
            layers.append(q.RY(qubit=w, theta=th, remapping=None))
            gates.append(("ry", w, th, None))
        for w in range(n - 1):
            th = float(np.float32(rng.uniform(0, 2 * np.pi)))
            k = ("rx", "ry", "rz")[(w + d) % 3]
            cls = {"rx": q.RX, "ry": q.RY, "rz": q.RZ}[k]
            c, t = (w, w + 1) if d % 2 == 0 else (w + 1, w)
            layers.append(q.Controlled(c, cls(qubit=t, theta=th, remapping=None)))
            gates.append(("c" + k, c, t, th, None))
        layers.append(q.Controlled(n - 1, q.RY(qubit=0, name="x", remapping=None)))
        gates.append(("cry", n - 1, 0, None, "x"))
        th = float(np.float32(rng.uniform(0, 2 * np.pi)))
        layers.append(q.Invert(q.RX(qubit=d, theta=th, remapping=None).build(num_qubits=n)))
        gates.append(("rx", d, -th, None))
        layers.append(q.Invert(q.CNOT(d, n - 1).build(num_qubits=n)))
        gates.append(("cnot", d, n - 1))
    layers.append(q.MeasureProbability())
    desc = {"n": n, "batch": batch, "gates": gates, "inputs": {"x": x}, "measure": "p0"}
    return layers, desc, {"x": x}


@pytest.mark.parametrize("compiled", [True, False], ids=["compiled", "interpreted"])
def test_mixed_circuit_fused_vs_oracle(cuda_device, compiled):
    layers, desc, inputs = _mixed()
    n, B = desc["n"], desc["batch"]
    circ = q.Circuit(layers, num_qubits=n, compiled=compiled).to(cuda_device)
    st = torch.zeros(B, 1 << n, dtype=torch.complex64, device=cuda_device)
    st[:, 0] = 1
    x = torch.tensor(inputs["x"], device=cuda_device, requires_grad=True)
    p0 = circ(st, x=x)
    ref = oracle.forward(desc, state=st.cpu().numpy())
    assert np.abs(p0.detach().cpu().numpy() - ref).max() < TOL
    w = torch.linspace(-1, 1, n, device=cuda_device)
    (p0 * w).sum().backward()
    rdth, rdn, _ = oracle.adjoint(desc, np.broadcast_to(w.cpu().numpy(), (B, n)).astype(np.float64), "p0",
                                  state=st.cpu().numpy())
    # module angles in gate order; an inverted rotation is the oracle's
    # rotation by the negated angle, so its gradient flips sign
    got = []
    for m in circ.circuit.layers:
        name = type(m).__name__
        if name in ("BuiltRY", "BuiltRX", "BuiltRZ"):
            got.append(float(m.theta.grad))
        elif name == "BuiltControlled" and not m.t.named:
            got.append(float(m.t.theta.grad))
        elif name == "BuiltInvert" and hasattr(m.target, "theta"):
            got.append(-float(m.target.theta.grad))
    got = np.array(got)
    assert got.shape == rdth.shape
    assert np.abs(got - rdth).max() < 1e-4
    assert np.abs(x.grad.cpu().numpy() - rdn["x"]).max() < 1e-4

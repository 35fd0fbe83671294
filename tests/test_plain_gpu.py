"""Plain form (one CUDA pass per gate) against the reference's golden vectors
and the complex128 oracle.  Mirrors the reference's sweeps
(test/test_operators.py:85-203, test_embeddings.py:56-153,
test_measurements.py:6-48, test_ansaetze.py:6-83)."""
import json

import numpy as np
import pytest
import torch

import qandle_gb300 as q
from oracle import oracle
from qandle_gb300 import workloads
from tests import golden_io

pytestmark = pytest.mark.gpu

TOL = 1e-5  # max-abs, complex64 engine vs complex64 reference / complex128 oracle


def _gate_module(gate, n):
    k = gate[0]
    if k in ("rx", "ry", "rz"):
        cls = {"rx": q.RX, "ry": q.RY, "rz": q.RZ}[k]
        return cls(qubit=gate[1], theta=torch.tensor(np.float32(gate[2])), remapping=None).build(n)
    if k == "u":
        return q.U(qubit=gate[1], matrix=torch.tensor(gate[2])).build(n)
    if k == "cnot":
        return q.CNOT(gate[1], gate[2]).build(n)
    if k == "cz":
        return q.CZ(gate[1], gate[2]).build(n)
    return q.SWAP(gate[1], gate[2]).build(n)


def test_gates_vs_reference(cuda_device):
    z = golden_io.load("gates")
    worst = 0.0
    for i in range(int(z["count"])):
        d = json.loads(str(z[f"g{i}_desc"]))
        gate = golden_io.parse_gate(d["gate"])
        mod = _gate_module(gate, d["n"]).to(cuda_device)
        inp = torch.tensor(z[f"g{i}_in"], device=cuda_device)
        out = mod(inp).detach().cpu().numpy()
        ref = z[f"g{i}_out"]
        assert out.shape == ref.shape
        if gate[0] in ("cnot", "cz", "swap"):
            assert np.array_equal(out, ref), (i, gate)  # exact moves / sign flips
        else:
            err = np.abs(out - ref).max()
            worst = max(worst, err)
            assert err < TOL, (i, gate, err)
            desc = {"n": d["n"], "batch": None, "gates": [gate], "inputs": {}}
            o = oracle.run(desc, state=z[f"g{i}_in"],
                           batch=z[f"g{i}_in"].shape[0] if z[f"g{i}_in"].ndim == 2 else 1)
            assert np.abs(out.reshape(o.shape) - o).max() < TOL
    print(f"max |engine - reference| over single gates: {worst:.2e}")


def test_embeddings_vs_reference(cuda_device):
    z = golden_io.load("embeddings")
    for i in range(int(z["count"])):
        d = json.loads(str(z[f"e{i}_desc"]))
        emb = q.AngleEmbedding(name="e", qubits=d["qubits"], rotation=d["rot"]).build(d["n"])
        x = torch.tensor(z[f"e{i}_x"], device=cuda_device)
        out = emb(e=x).detach().cpu().numpy()
        ref = z[f"e{i}_out"]
        assert out.shape == ref.shape
        assert np.abs(out - ref).max() < TOL, i


def test_measurements_vs_reference(cuda_device):
    z = golden_io.load("measurements")
    for i in range(int(z["count"])):
        inp = torch.tensor(z[f"m{i}_in"], device=cuda_device)
        n = inp.shape[-1].bit_length() - 1
        p0 = q.MeasureProbabilityBuilt(num_qubits=n)(inp).detach().cpu().numpy()
        ref = z[f"m{i}_p0"]
        assert p0.shape == ref.shape, (i, p0.shape, ref.shape)  # the reference's squeeze quirks
        assert np.abs(p0 - ref).max() < TOL
        pj = q.MeasureJointProbability()(inp).detach().cpu().numpy()
        assert pj.shape == z[f"m{i}_joint"].shape
        assert np.abs(pj - z[f"m{i}_joint"]).max() < TOL


def test_sel_vs_reference(cuda_device):
    z = golden_io.load("sel")
    for i in range(int(z["count"])):
        d = json.loads(str(z[f"s{i}_desc"]))
        sel = q.StronglyEntanglingLayer(qubits=list(range(d["n"])), depth=d["depth"],
                                        q_params=torch.tensor(z[f"s{i}_w"]), remapping=None)
        mod = sel.build(num_qubits=d["n"]).to(cuda_device)
        out = mod(torch.tensor(z[f"s{i}_in"], device=cuda_device)).detach().detach().cpu().numpy()
        assert np.abs(out - z[f"s{i}_out"]).max() < TOL, i


def test_reupload_vs_reference(cuda_device):
    z = golden_io.load("reupload")
    c2 = q.Circuit([q.RX(qubit=1, name="reupload", remapping=None)], num_qubits=3,
                   engine="plain").to(cuda_device)
    dev = lambda a: torch.tensor(a, device=cuda_device)  # noqa: E731
    v, vb = dev(z["v"]), dev(z["vb"])
    for got, ref in ((c2(dev(z["inp_u"]), reupload=v), z["unb"]),
                     (c2(dev(z["inp_b"]), reupload=v), z["bat_scalar"]),
                     (c2(dev(z["inp_b"]), reupload=vb), z["bat_vec"]),
                     (c2(dev(z["inp_u"]), reupload=vb), z["unb_vec"])):
        got = got.detach().detach().cpu().numpy()
        assert got.shape == ref.shape
        assert np.abs(got - ref).max() < TOL


@pytest.mark.parametrize("name", ["plain_small", "sel_small", "deep_small"])
def test_circuits_plain_vs_reference(cuda_device, name):
    z = golden_io.load("circuits")
    desc = golden_io.circuit_desc(z, name)
    if desc["measure"] == "z":
        desc["measure"] = "p0"  # the golden file holds MeasureProbability
    circ = workloads.build_circuit(desc, engine="plain").to(cuda_device)
    kw = workloads.circuit_inputs(desc, cuda_device)
    if name == "deep_small":
        st = torch.zeros(desc["batch"], 1 << desc["n"], dtype=torch.complex64, device=cuda_device)
        st[:, 0] = 1
        out = circ(st)
    else:
        out = circ(**kw)
    out = out.detach().detach().cpu().numpy()
    ref = z[f"{name}_out"]
    assert out.shape == ref.shape
    assert np.abs(out - ref).max() < TOL
    o = oracle.forward(desc)
    assert np.abs(out.reshape(o.shape) - o).max() < TOL


def test_plain_autograd_vs_reference(cuda_device):
    """Per-layer autograd through the plain kernels equals qandle's torch
    autograd (golden) on the adjoint-brick family."""
    z = golden_io.load("circuits")
    desc = golden_io.circuit_desc(z, "brick_small")
    desc["measure"] = "p0"
    circ = workloads.build_circuit(desc, engine="plain").to(cuda_device)
    st = torch.zeros(desc["batch"], 1 << desc["n"], dtype=torch.complex64, device=cuda_device)
    st[:, 0] = 1
    p0 = circ(st)
    zexp = 2.0 * p0 - 1.0
    loss = ((zexp - torch.tensor(desc["targets"], device=cuda_device)) ** 2).mean()
    loss.backward()
    grads = [m.theta.grad.item() for m in circ.circuit.layers
             if isinstance(m, q.BuiltParametrizedOperator)]
    assert abs(loss.item() - float(z["brick_small_loss"])) < 1e-5
    assert np.abs(np.array(grads) - z["brick_small_dtheta"]).max() < 1e-5


def test_plain_embedding_grad_vs_reference(cuda_device):
    z = golden_io.load("circuits")
    desc = golden_io.circuit_desc(z, "sel_small")
    desc["measure"] = "p0"
    circ = workloads.build_circuit(desc, engine="plain").to(cuda_device)
    x = torch.tensor(desc["inputs"]["x"], device=cuda_device, requires_grad=True)
    kw = {"x": x}
    for qq in range(desc["n"]):
        kw[f"up{qq}"] = x[:, qq]
    p0 = circ(**kw)
    (p0 * torch.tensor(z["sel_small_weights"], device=cuda_device)).sum().backward()
    grads = [m.theta.grad.item() for m in circ.circuit.layers
             if isinstance(m, q.BuiltParametrizedOperator) and not m.named]
    assert np.abs(np.array(grads) - z["sel_small_dtheta"]).max() < 1e-5
    assert np.abs(x.grad.cpu().numpy() - z["sel_small_dx"]).max() < 1e-5


def test_plain_edge_cases(cuda_device):
    # one qubit, unbatched and batched
    for shape in ((2,), (3, 2)):
        st = torch.randn(*shape, dtype=torch.complex64, device=cuda_device)
        for k in ("rx", "ry", "rz"):
            g = (k, 0, 0.7, None)
            out = _gate_module(g, 1).to(cuda_device)(st).detach().cpu().numpy()
            o = oracle.run({"n": 1, "batch": None, "gates": [g], "inputs": {}},
                           state=st.cpu().numpy(), batch=st.reshape(-1, 2).shape[0])
            assert np.abs(out.reshape(o.shape) - o).max() < TOL
    # SWAP of a qubit with itself is the identity (operators.py:661-671)
    st = torch.randn(4, 8, dtype=torch.complex64, device=cuda_device)
    assert torch.equal(q.SWAP(1, 1).build(3).to(cuda_device)(st), st)
    # errors: out-of-range qubit, CPU tensors
    with pytest.raises(RuntimeError):
        q.RX(5, theta=0.1, remapping=None).build(3).to(cuda_device)(st)
    with pytest.raises(RuntimeError):
        q.RX(0, theta=0.1, remapping=None).build(3)(st.cpu())

"""Front-end layers on the GPU against the reference's outputs:

* AmplitudeEmbedding with more features than 2^n and a pad value cuts the
  features past 2^n as the reference does (tests/golden/amplitude_crop.npz);
* a circuit with nested circuits, run for inference (the per-gate in-place
  path), equals its decomposition;
* TwoLocal, SU and the budget ansatz, on the fused engine (6 qubits) and the
  per-gate kernels (4 qubits), give the reference's states
  (tests/golden/ansaetze.npz);
* split circuits, moved to the GPU (their gates on the parent qubits share
  the subcircuits' parameters), give the reference's split states
  (tests/golden/splitter.npz), on the fused engine and, at 3 qubits, the
  per-gate kernels.
"""
import json

import numpy as np
import pytest
import torch

import qandle_gb300 as q
from tests import golden_io
from tests.golden import make_golden as mg

pytestmark = pytest.mark.gpu
DEV = "cuda"


def test_amplitude_crop_matches_reference():
    z = golden_io.load("amplitude_crop")
    for i in range(int(z["count"])):
        spec = json.loads(str(z[f"c{i}_spec"]))
        x = torch.tensor(z[f"c{i}_x"], device=DEV)
        emb = q.AmplitudeEmbedding(name="x", qubits=list(range(spec["n"])), normalize=spec["normalize"],
                                   pad_with=spec["pad"]).build(num_qubits=spec["n"])
        err = float(np.abs(emb(x=x).cpu().numpy() - z[f"c{i}_out"]).max())
        assert err < 1e-6, (spec, err)


def test_nested_circuit_inference_equals_decomposition():
    n = 3
    c1 = q.Circuit([q.RX(0, theta=0.3, remapping=None), q.CNOT(0, 1)], num_qubits=n)
    c2 = q.Circuit([q.RY(1, theta=-0.8, remapping=None), q.StronglyEntanglingLayer(qubits=[1, 2], remapping=None)],
                   num_qubits=n)
    outer = q.Circuit([c1, q.RZ(0, theta=1.1, remapping=None), c2, q.CNOT(2, 0)], num_qubits=n).to(DEV)
    flat = outer.decompose().to(DEV)
    psi = torch.randn(4, 1 << n, dtype=torch.cfloat, generator=torch.Generator().manual_seed(0))
    psi = (psi / psi.norm(dim=1, keepdim=True)).to(DEV)
    with torch.no_grad():
        a = outer(psi)
    b = flat(psi).detach()
    assert float((a - b).abs().max()) < 1e-5


@pytest.mark.parametrize("name", ["twolocal_6", "su_6", "budget_6", "twolocal_full", "su_full"])
def test_ansatz_state_matches_reference(name):
    z = golden_io.load("ansaetze")
    kind, nq, args = mg.ansatz_circuits()[name]
    circ = mg.build_ansatz(q, kind, nq, args)
    rec = json.loads(str(z[name]))
    with torch.no_grad():
        for p, v in zip(circ.parameters(), rec["params"]):
            p.fill_(v)
    for m in circ.circuit.layers[0].applied_gates:  # the fixtures use the identity remapping
        if hasattr(m, "remapping"):
            m.remapping = q.remap.none
    circ = circ.to(DEV)
    rng = np.random.default_rng(11)
    ps = rng.normal(size=(1 << nq,)) + 1j * rng.normal(size=(1 << nq,))
    ps = torch.tensor(ps / np.linalg.norm(ps), dtype=torch.cfloat, device=DEV)
    ref = z[name + "_state"].reshape(-1)
    for grad in ((False, True) if nq < 5 else (False,)):
        with torch.set_grad_enabled(grad):
            st = circ(ps)
        err = float(np.abs(st.detach().cpu().numpy().reshape(-1) - ref).max())
        assert err < 2e-6, (grad, err)


@pytest.mark.parametrize("name", ["cnot10_k5", "sel6_k3", "random1_k3", "random2_k3", "dummy_k2"])
def test_split_circuit_state_matches_reference(name):
    z = golden_io.load("splitter")
    gates, n, k, via = mg.split_circuits()[name]
    split = mg.build_split(q, gates, n, k, via)
    for la in split.circuit.layers:  # the fixture's states use the identity remapping
        if hasattr(la, "remapping"):
            la.remapping = q.remap.none
    split = split.to(DEV)
    psi, named = mg.split_inputs(n, gates)
    kw = {nm: torch.tensor(v, dtype=torch.float32, device=DEV) for nm, v in named.items()}
    with torch.no_grad():
        st = split(torch.tensor(psi, dtype=torch.cfloat, device=DEV), **kw)
    ref = np.asarray(z[name + "_state"]).reshape(-1)
    err = float(np.abs(st.cpu().numpy().reshape(-1) - ref).max())
    assert err < 2e-6, err

"""Fused engine on the GPU against the reference's golden vectors and the
complex128 oracle: forward (every measurement kind, several tile shapes,
n below and above the tile size, partial tiles) and the adjoint backward
(shared angles, named inputs, embedding inputs, input-state gradient,
checkpoint segments)."""
import numpy as np
import pytest
import torch

import qandle_gb300 as q
from oracle import oracle
from qandle_gb300 import workloads
from tests import golden_io

pytestmark = pytest.mark.gpu

TOL = 1e-5    # max-abs on probabilities / P0 / <Z> / amplitudes
GTOL = 1e-4   # max-abs on gradients (sums over up to 2^n * batch terms in float32)


def _run(desc, dev, engine="fused", state=None, **opt):
    circ = workloads.build_circuit(desc, engine=engine, **opt).to(dev)
    kw = workloads.circuit_inputs(desc, dev)
    with torch.no_grad():
        out = circ(state, **kw) if state is not None else circ(**kw)
    return out.detach().cpu().numpy()


@pytest.mark.parametrize("name", ["plain_small", "sel_small", "deep_small"])
def test_fused_vs_reference_golden(cuda_device, name):
    z = golden_io.load("circuits")
    desc = golden_io.circuit_desc(z, name)
    if desc["measure"] == "z":
        desc["measure"] = "p0"
    st = None
    if name == "deep_small":
        st = torch.zeros(desc["batch"], 1 << desc["n"], dtype=torch.complex64, device=cuda_device)
        st[:, 0] = 1
    out = _run(desc, cuda_device, state=st)
    ref = z[f"{name}_out"]
    assert out.shape == ref.shape
    assert np.abs(out - ref).max() < TOL


CASES = {
    "sel_n10": lambda: workloads.sel_reupload(n=10, batch=37, layers=3, reupload_every=2),
    "sel_n14": lambda: workloads.sel_reupload(n=14, batch=3, layers=4, reupload_every=2),
    "sel_n16": lambda: workloads.sel_reupload(n=16, batch=2, layers=3, reupload_every=2, measure="p0"),
    "brick_n15": lambda: workloads.adjoint_brick(n=15, batch=3, layers=6),
    "deep_n15": lambda: workloads.deep_u(n=15, batch=2, layers=5),
    "plain_n5": lambda: workloads.plain_small(n=5, batch=300, layers=3),
    "plain_n8": lambda: workloads.plain_small(n=8, batch=64, layers=4),
    "plain_n12": lambda: workloads.plain_small(n=12, batch=5, layers=3),
}
OPTS = [dict(), dict(tile_bits=12, low_bits=4, max_high=2), dict(tile_bits=11, low_bits=5, max_high=1),
        dict(tile_bits=13, low_bits=7, max_high=6), dict(reg_bits=4), dict(tile_bits=12, reg_bits=4),
        dict(max_high=5, reg_search=1)]


@pytest.mark.parametrize("compiled", [True, False], ids=["compiled", "interpreted"])
@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("oi", range(len(OPTS)))
def test_fused_forward_vs_oracle(cuda_device, case, oi, compiled):
    desc = CASES[case]()
    out = _run(desc, cuda_device, compiled=compiled, **OPTS[oi])
    ref = oracle.forward(desc)
    if out.shape == ref.shape[1:]:
        ref = ref[0]  # no per-sample input: the front end runs the unbatched |0..0> state
    err = np.abs(out - ref).max()
    assert err < TOL, (case, OPTS[oi], err)


def test_compiled_backward_kernels_run(cuda_device):
    """A training call compiles the backward passes too and runs them."""
    desc = workloads.adjoint_brick(n=12, batch=2, layers=3)
    desc["measure"] = "p0"
    circ = workloads.build_circuit(desc, engine="fused").to(cuda_device)
    st = torch.zeros(2, 1 << 12, dtype=torch.complex64, device=cuda_device)
    st[:, 0] = 1
    circ(st).sum().backward()
    prog = circ._executor.program(True)
    assert prog.keep_state and prog.compiled(cuda_device)


def test_compiled_kernels_run(cuda_device):
    """The default forward runs the per-program compiled pass kernels."""
    desc = workloads.sel_reupload(n=14, batch=3, layers=2, reupload_every=2)
    circ = workloads.build_circuit(desc, engine="fused").to(cuda_device)
    with torch.no_grad():
        circ(**workloads.circuit_inputs(desc, cuda_device))
    assert circ._executor.compiled
    assert circ._executor.program(False).compiled(cuda_device)


@pytest.mark.parametrize("reg_bits", [5, 4])
def test_headline_circuit_full_width(cuda_device, reg_bits):
    """The benchmark circuit itself (20 qubits, 10 SEL layers, re-uploads,
    <Z>) at batch 2, compiled, against the oracle."""
    desc = workloads.sel_reupload(n=20, batch=2)
    out = _run(desc, cuda_device, reg_bits=reg_bits)
    ref = oracle.forward(desc)
    assert np.abs(out - ref).max() < TOL


@pytest.mark.parametrize("measure", ["state", "probs", "p0", "z"])
def test_fused_measure_kinds(cuda_device, measure):
    desc = workloads.sel_reupload(n=14, batch=3, layers=2, reupload_every=2, measure=measure)
    out = _run(desc, cuda_device)
    ref = oracle.forward(desc)
    assert out.shape == ref.shape
    assert np.abs(out - ref).max() < TOL


def test_fused_unbatched_and_input_state(cuda_device):
    desc = workloads.adjoint_brick(n=13, batch=1, layers=3)
    desc["measure"] = "state"
    g = torch.Generator().manual_seed(5)
    st = torch.randn(1 << 13, generator=g, dtype=torch.complex64)
    st = st / st.abs().pow(2).sum().sqrt()
    out = _run(desc, cuda_device, state=st.to(cuda_device))
    assert out.shape == (1 << 13,)
    ref = oracle.run(desc, state=st.numpy(), batch=1)[0]
    assert np.abs(out - ref).max() < TOL


def _grad_case(desc, dev, opts, weights_seed=3):
    circ = workloads.build_circuit(desc, engine="fused", **opts).to(dev)
    x = None
    kw = {}
    if "x" in desc["inputs"]:
        x = torch.tensor(desc["inputs"]["x"], device=dev, requires_grad=True)
        kw["x"] = x
        for qq in range(desc["n"]):
            if f"up{qq}" in desc["inputs"]:
                kw[f"up{qq}"] = x[:, qq]
    if x is None:  # batched |0..0> input so every sample has its own row
        st = torch.zeros(desc["batch"], 1 << desc["n"], dtype=torch.complex64, device=dev)
        st[:, 0] = 1
        out = circ(st, **kw)
    else:
        out = circ(**kw)
    g = torch.Generator().manual_seed(weights_seed)
    w = torch.rand(out.shape, generator=g).to(dev) * 2 - 1
    (out * w).sum().backward()
    thetas = [m.theta.grad.item() for m in circ.circuit.layers
              if isinstance(m, q.BuiltParametrizedOperator) and not m.named]
    return np.array(thetas), (x.grad.cpu().numpy() if x is not None else None), w.cpu().numpy()


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("oi", [0, 1, 4, 6])
def test_compiled_equals_interpreted_bitwise(cuda_device, case, oi):
    """The compiled pass kernels and the op interpreter run the same op list
    with the same pending-X rules and arithmetic: identical bits (the
    serving loop moves a request between them at a pass boundary)."""
    desc = CASES[case]()
    a = _run(desc, cuda_device, compiled=True, **OPTS[oi])
    b = _run(desc, cuda_device, compiled=False, **OPTS[oi])
    assert np.array_equal(a, b), (case, OPTS[oi], np.abs(a - b).max())


@pytest.mark.parametrize("case,opts", [
    ("brick_n10", dict()), ("brick_n14", dict()), ("brick_n16", dict(checkpoint_segments=3)),
    ("sel_n9", dict()), ("sel_n14", dict(checkpoint_segments=2)), ("sel_n15", dict(tile_bits=12, low_bits=4)),
    ("brick_n13", dict(reg_bits=4)), ("sel_n8", dict(reg_bits=4, checkpoint_segments=2)),
])
@pytest.mark.parametrize("compiled", [True, False], ids=["compiled", "interpreted"])
def test_fused_adjoint_vs_oracle(cuda_device, case, opts, compiled):
    opts = dict(opts, compiled=compiled)
    kind, nq = case.split("_n")
    n = int(nq)
    if kind == "brick":
        desc = workloads.adjoint_brick(n=n, batch=4, layers=5)
        desc["measure"] = "p0"
    else:
        desc = workloads.sel_reupload(n=n, batch=3, layers=3, reupload_every=2, measure="p0")
    dth, dx, w = _grad_case(desc, cuda_device, opts)
    rdp, rdn, _ = oracle.adjoint(desc, w, "p0")
    assert np.abs(dth - rdp).max() < GTOL, np.abs(dth - rdp).max()
    if dx is not None:
        ref = rdn["x"].copy()
        for qq in range(n):
            ref[:, qq] += rdn[f"up{qq}"]
        assert np.abs(dx - ref).max() < GTOL


def test_fused_adjoint_vs_reference_autograd(cuda_device):
    """MSE(<Z>, targets) on the adjoint-brick family equals qandle's own torch
    autograd gradient (golden)."""
    z = golden_io.load("circuits")
    desc = golden_io.circuit_desc(z, "brick_small")
    desc["measure"] = "p0"
    circ = workloads.build_circuit(desc, engine="fused").to(cuda_device)
    st = torch.zeros(desc["batch"], 1 << desc["n"], dtype=torch.complex64, device=cuda_device)
    st[:, 0] = 1
    p0 = circ(st)
    zexp = 2.0 * p0 - 1.0
    loss = ((zexp - torch.tensor(desc["targets"], device=cuda_device)) ** 2).mean()
    loss.backward()
    grads = [m.theta.grad.item() for m in circ.circuit.layers if isinstance(m, q.BuiltParametrizedOperator)]
    assert abs(loss.item() - float(z["brick_small_loss"])) < 1e-5
    assert np.abs(np.array(grads) - z["brick_small_dtheta"]).max() < 1e-5


def test_fused_state_gradient(cuda_device):
    desc = workloads.adjoint_brick(n=11, batch=2, layers=2)
    desc["measure"] = "probs"
    circ = workloads.build_circuit(desc, engine="fused").to(cuda_device)
    g = torch.Generator().manual_seed(9)
    st0 = torch.randn(2, 1 << 11, generator=g, dtype=torch.complex64)
    st = st0.to(cuda_device).requires_grad_(True)
    out = circ(st)
    w = torch.rand(out.shape, generator=g).to(cuda_device)
    (out * w).sum().backward()
    _, _, dps = oracle.adjoint(desc, w.cpu().numpy(), "probs", state=st0.numpy())
    assert np.abs(st.grad.cpu().numpy() - dps).max() < GTOL


def test_fused_matches_plain(cuda_device):
    desc = workloads.sel_reupload(n=13, batch=4, layers=3, reupload_every=2)
    a = _run(desc, cuda_device, engine="fused")
    b = _run(desc, cuda_device, engine="plain")
    assert np.abs(a - b).max() < TOL


def test_deep_28_qubits(cuda_device):
    """The 28-qubit, batch-1 deep circuit (50 layers of U with CNOT+SWAP
    brickwork, 2 GiB state): the full run keeps the norm and agrees with the
    per-gate form; the same circuit restricted to qubits 0..19 matches the
    complex128 oracle."""
    desc = workloads.deep_u(n=28, batch=1, layers=50)
    circ = workloads.build_circuit(desc, engine="fused").to(cuda_device)
    with torch.no_grad():
        probs = circ().reshape(-1)
    assert abs(float(probs.double().sum()) - 1.0) < 1e-4
    circ_p = workloads.build_circuit(desc, engine="plain").to(cuda_device)
    with torch.no_grad():
        probs_p = circ_p().reshape(-1)
    assert float((probs - probs_p).abs().max()) < TOL
    del probs, probs_p
    pre = workloads.restrict(desc, 20)
    out = _run(pre, cuda_device)
    ref = oracle.forward(pre)
    if out.shape == ref.shape[1:]:
        ref = ref[0]
    assert np.abs(out - ref).max() < TOL


def test_autotune_on_device(cuda_device, tmp_path):
    """Circuit.tune times real candidate plans, keeps the fastest, and the
    tuned circuit still matches the oracle."""
    desc = workloads.sel_reupload(n=14, batch=8, layers=2, reupload_every=2)
    circ = workloads.build_circuit(desc, engine="fused").to(cuda_device)
    cands = [dict(tile_bits=13, low_bits=6), dict(tile_bits=12, low_bits=6)]
    res = circ.tune(8, cuda_device, candidates=cands, cache_path=str(tmp_path / "tune.json"))
    assert res["options"] in cands and res["ms"] > 0 and len(res["timings"]) == 2
    with torch.no_grad():
        out = circ(**workloads.circuit_inputs(desc, cuda_device)).cpu().numpy()
    assert np.abs(out - oracle.forward(desc)).max() < TOL

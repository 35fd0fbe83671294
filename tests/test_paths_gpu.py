"""GPU paths that the forward/adjoint tests do not reach on their own:

* the captured forward: BoundForward.capture/replay, and Circuit.__call__,
  which replays one captured CUDA graph per (device, batch, input kind) on
  inference calls -- against the complex128 oracle, on repeated calls with new
  inputs, and bit-identical to the uncaptured launch;
* the adjoint workload at its full depth (16 qubits, 20 layers of RX RY with
  CZ/CNOT bricks, 640 angles, MSE(<Z>, targets), four checkpoint segments) on a
  few samples, against the oracle's adjoint gradient;
* an OpenQASM 3 request (the serving wire format) through the serving loop,
  against the oracle;
* the per-circuit binding a qandle maintainer adds (FusedExecutor injected
  into a circuit of the reference's own classes), against the reference's
  torch forward and autograd.
"""
import numpy as np
import pytest
import torch

import qandle_gb300 as q
from oracle import oracle
from qandle_gb300 import engine, serve, workloads

pytestmark = pytest.mark.gpu

TOL = 1e-5    # max-abs on probabilities / P0 / <Z>
GTOL = 1e-4   # max-abs on gradients


def _inputs_seeded(desc, seed):
    """The description's named inputs redrawn from `seed` (x ~ U(0, pi), the
    re-upload columns follow x)."""
    d = dict(desc)
    g = torch.Generator().manual_seed(seed)
    x = (torch.rand(desc["batch"], desc["n"], generator=g) * np.pi).numpy().astype(np.float32)
    inputs = {"x": x}
    for k in desc["inputs"]:
        if k.startswith("up"):
            inputs[k] = np.ascontiguousarray(x[:, int(k[2:])])
    d["inputs"] = inputs
    return d


def test_bound_forward_graph_replay_vs_oracle(cuda_device):
    desc = workloads.sel_reupload(n=14, batch=5, layers=3, reupload_every=2)
    circ = workloads.build_circuit(desc, engine="fused", graphs=False).to(cuda_device)
    with torch.no_grad():
        circ(**workloads.circuit_inputs(desc, cuda_device))
    bound = engine.BoundForward(circ._executor, desc["batch"], cuda_device)
    bound.set_inputs(**workloads.circuit_inputs(desc, cuda_device))
    bound.capture()
    for seed in (1, 2):
        d = _inputs_seeded(desc, seed)
        bound.set_inputs(**workloads.circuit_inputs(d, cuda_device))
        bound.replay()
        torch.cuda.synchronize()
        out = bound.result().cpu().numpy()
        ref = oracle.forward(d)
        assert np.abs(out - ref).max() < TOL, seed


@pytest.mark.parametrize("measure", ["z", "p0", "probs"])
def test_circuit_call_replays_graph(cuda_device, measure):
    """Inference calls through the public API run a captured graph; new
    inputs at the same batch reuse it, a new batch captures another, and the
    results equal the oracle and, bit for bit, the uncaptured launch."""
    desc = workloads.sel_reupload(n=13, batch=4, layers=3, reupload_every=2, measure=measure)
    circ = workloads.build_circuit(desc, engine="fused").to(cuda_device)
    plain = workloads.build_circuit(desc, engine="fused", graphs=False).to(cuda_device)
    plain.load_state_dict(circ.state_dict())
    for seed in (3, 4):
        d = _inputs_seeded(desc, seed)
        kw = workloads.circuit_inputs(d, cuda_device)
        with torch.no_grad():
            out = circ(**kw)
            ref_launch = plain(**kw)
        assert torch.equal(out, ref_launch)
        assert np.abs(out.cpu().numpy() - oracle.forward(d)).max() < TOL
    ex = circ._executor
    assert len(ex._bounds) == 1
    (b,) = ex._bounds.values()
    assert b.graph is not None
    first = b
    # another batch size: a second captured forward beside the first
    d2 = dict(_inputs_seeded(desc, 5))
    d2["batch"] = 7
    d2 = _inputs_seeded(d2, 5)
    with torch.no_grad():
        out2 = circ(**workloads.circuit_inputs(d2, cuda_device))
    assert np.abs(out2.cpu().numpy() - oracle.forward(d2)).max() < TOL
    assert len(ex._bounds) == 2 and first in ex._bounds.values()


def test_circuit_call_graph_with_input_state(cuda_device):
    """An input state goes into the captured forward's static state buffer."""
    desc = workloads.adjoint_brick(n=12, batch=3, layers=4)
    desc["measure"] = "p0"
    circ = workloads.build_circuit(desc, engine="fused").to(cuda_device)
    g = torch.Generator().manual_seed(8)
    for _ in range(2):
        st = torch.randn(3, 1 << 12, generator=g, dtype=torch.complex64)
        st = st / st.abs().pow(2).sum(-1, keepdim=True).sqrt()
        with torch.no_grad():
            out = circ(st.to(cuda_device))
        ref = oracle.forward(desc, state=st.numpy())
        assert np.abs(out.cpu().numpy() - ref).max() < TOL
    assert any(b.graph is not None for b in circ._executor._bounds.values())


def test_training_call_does_not_use_graph(cuda_device):
    desc = workloads.adjoint_brick(n=12, batch=2, layers=2)
    desc["measure"] = "p0"
    circ = workloads.build_circuit(desc, engine="fused").to(cuda_device)
    st = torch.zeros(2, 1 << 12, dtype=torch.complex64, device=cuda_device)
    st[:, 0] = 1
    circ(st).sum().backward()
    assert not circ._executor._bounds
    assert all(m.theta.grad is not None for m in circ.circuit.layers if isinstance(m, q.BuiltParametrizedOperator))


def test_adjoint_workload_full_depth_vs_oracle(cuda_device):
    """The 16-qubit, 20-layer adjoint workload (640 angles, four checkpoint
    segments) at batch 4: loss and every angle's gradient against the oracle's
    complex128 adjoint of the same MSE(<Z>, targets)."""
    desc = workloads.adjoint_brick(n=16, batch=4, layers=20)
    desc["measure"] = "p0"
    n, B = desc["n"], desc["batch"]
    targets = torch.tensor(desc["targets"], device=cuda_device)
    circ = workloads.build_circuit(desc, engine="fused", checkpoint_segments=4).to(cuda_device)
    st = torch.zeros(B, 1 << n, dtype=torch.complex64, device=cuda_device)
    st[:, 0] = 1
    p0 = circ(st)
    loss = ((2.0 * p0 - 1.0 - targets) ** 2).mean()
    loss.backward()
    dth = np.array([m.theta.grad.item() for m in circ.circuit.layers
                    if isinstance(m, q.BuiltParametrizedOperator)])
    assert dth.size == 640
    p0_ref = oracle.forward(desc)
    loss_ref, gp0 = oracle.mse_z_grad(2.0 * p0_ref - 1.0, desc["targets"].astype(np.float64))
    assert abs(loss.item() - loss_ref) < TOL
    rdp, _, _ = oracle.adjoint(desc, gp0, "p0")
    err = np.abs(dth - rdp).max()
    assert err < GTOL, err


def test_qasm_request_through_server(cuda_device):
    """A circuit exported as OpenQASM 3 (AngleEmbedding and re-uploads as
    named rx inputs), read back by serve.description_from_qasm and served
    next to an ordinary request: its <Z> equals the oracle's."""
    desc = workloads.sel_reupload(n=9, batch=6, layers=4, reupload_every=2)
    text = workloads.build_circuit(desc).to_openqasm3()
    x = desc["inputs"]["x"]
    inputs = {}
    for line in text.splitlines():
        if line.startswith("input float "):
            name = line[len("input float "):-1]
            col = int(name[2:]) if name.startswith("up") else int(name.rsplit("_", 1)[1])
            inputs[name] = x[:, col]
    req = serve.description_from_qasm(text, inputs, batch=desc["batch"], measure="z")
    other = workloads.sel_reupload(n=12, batch=3, layers=2, reupload_every=2)
    srv = serve.Server(cuda_device, hbm_budget=1 << 30)
    try:
        h_other = srv.submit(other)
        h = srv.submit(req)
        out = h.future.result(timeout=120)
        out_other = h_other.future.result(timeout=120)
    finally:
        srv.close()
    assert np.abs(out.numpy() - oracle.forward(desc)).max() < TOL
    assert np.abs(out_other.numpy() - oracle.forward(other)).max() < TOL


def test_integration_snippet_on_reference_circuit(cuda_device):
    """The per-circuit binding as a qandle maintainer writes it, on a circuit built from the
    reference's own classes (qandle 0.1.8 installed in baseline/_ref): the
    fused forward equals the reference's torch forward on the CPU, and the
    adjoint gradients equal the reference's torch autograd gradients."""
    from oracle import reference_torch as rt

    why = rt.unavailable_reason()
    if why:
        pytest.skip(why)
    qandle = rt.import_reference()
    desc = workloads.sel_reupload(n=10, batch=4, layers=3, reupload_every=2, measure="p0")
    kw_cpu = rt.inputs(desc)
    ref_circ = rt.build_circuit(qandle, desc)
    want = ref_circ(**kw_cpu)
    want.sum().backward()
    want_grads = [m.theta.grad.clone() for m in ref_circ.circuit.layers
                  if hasattr(m, "theta") and not m.named]

    circ = rt.build_circuit(qandle, desc).to(cuda_device)  # qandle's own classes
    fused = engine.FusedExecutor(circ.circuit)              # lowers circ.circuit.layers once
    circ.circuit.forward = lambda state=None, **kw: fused(state, **kw)
    kw = {k: v.to(cuda_device) for k, v in kw_cpu.items()}
    out = circ(**kw)                                        # fused forward
    assert np.abs(out.detach().cpu().numpy() - want.detach().numpy()).max() < TOL
    out.sum().backward()                                    # adjoint backward
    got = [m.theta.grad for m in circ.circuit.layers if hasattr(m, "theta") and not m.named]
    assert len(got) == len(want_grads) > 0
    err = max(float((g.cpu() - w).abs().max()) for g, w in zip(got, want_grads))
    assert err < TOL, err


def test_fp32_probe_counts_its_fmas(cuda_device):
    """The FP32 roof probe launches one block of 256 threads per quarter SM
    and reports the FMAs it performed (8 chains x 2 lanes per iteration)."""
    import ctypes

    from qandle_gb300 import _lib

    lib = _lib.load()
    blocks = lib.qg_fp32_probe_blocks()
    assert blocks == 4 * torch.cuda.get_device_properties(cuda_device).multi_processor_count
    out = torch.zeros(blocks, dtype=torch.float32, device=cuda_device)
    cnt = ctypes.c_int64()
    _lib.check(lib.qg_fp32_probe(out.data_ptr(), blocks, 64, ctypes.byref(cnt), _lib.stream()))
    torch.cuda.synchronize()
    assert cnt.value == blocks * 256 * 64 * 16
    assert torch.isfinite(out).all() and (out != 0).all()
    # too small an output buffer is refused before launch
    assert lib.qg_fp32_probe(out.data_ptr(), blocks - 1, 64, ctypes.byref(cnt), _lib.stream()) != 0


def test_timed_backward_records_every_pass(cuda_device):
    """The adjoint with pass events gives the same gradients as without, and
    an event pair around each backward pass."""
    desc = workloads.adjoint_brick(n=14, batch=4, layers=4)
    desc["measure"] = "p0"
    circ = workloads.build_circuit(desc, engine="fused").to(cuda_device)
    st = torch.zeros(4, 1 << 14, dtype=torch.complex64, device=cuda_device)
    st[:, 0] = 1
    circ(st).sum().backward()
    params = [m.theta for m in circ.circuit.layers if isinstance(m, q.BuiltParametrizedOperator)]
    g0 = torch.stack([p.grad.reshape(()) for p in params]).clone()
    for p in params:
        p.grad = None
    ex = circ._executor
    nb = ex.program(True).info.backward_passes
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(2 * nb)]
    ex.backward_events = evs
    circ(st).sum().backward()
    torch.cuda.synchronize()
    assert ex.backward_events is None  # used by one backward
    g1 = torch.stack([p.grad.reshape(()) for p in params])
    assert torch.equal(g0, g1)
    ms = [evs[2 * i].elapsed_time(evs[2 * i + 1]) for i in range(nb)]
    assert all(m >= 0 for m in ms) and sum(ms) > 0


def test_first_graph_call_multi_pass_with_input_state(cuda_device):
    """The first inference call captures the graph; its warm-up launch
    advances the static state of a plan with several passes, and the call's
    input state must go in again before the replay (an 8-qubit circuit
    planned into 11 passes)."""
    desc = workloads.deep_u(n=8, batch=3, layers=6)
    circ = workloads.build_circuit(desc, engine="fused", fwd_max_mats=4).to(cuda_device)
    st = torch.zeros(3, 1 << 8, dtype=torch.complex64, device=cuda_device)
    st[:, 0] = 1
    ref = oracle.forward(desc)
    for _ in range(2):  # the capturing call and a replay
        with torch.no_grad():
            out = circ(st)
        assert circ._executor.program(False).info.forward_passes > 1
        assert np.abs(out.cpu().numpy() - ref).max() < TOL


def test_small_calls_plan_uncapped_passes(cuda_device):
    """With the default pass length, a call whose passes have fewer tiles
    than the GPU has SMs runs the uncapped plan (one pass for this 13-qubit,
    12-layer circuit), a larger call the capped one; both give the oracle's
    <Z>."""
    sms = torch.cuda.get_device_properties(cuda_device).multi_processor_count
    for batch, one_pass in ((4, True), (2 * sms, False)):
        desc = workloads.sel_reupload(n=13, batch=batch, layers=12, reupload_every=4)
        circ = workloads.build_circuit(desc, engine="fused").to(cuda_device)
        with torch.no_grad():
            out = circ(**workloads.circuit_inputs(desc, cuda_device))
        passes = circ._executor.program(False).info.forward_passes
        assert (passes == 1) == one_pass, (batch, passes)
        ref = oracle.forward(dict(desc, batch=min(batch, 8),
                                  inputs={k: v[:8] for k, v in desc["inputs"].items()}))
        assert np.abs(out[:8].cpu().numpy() - ref).max() < TOL

"""Fusion planner on the CPU: planned programs, executed by the op emulator
(tests/program_emulator.py), equal the complex128 oracle.  Covers tile
selection, commutation reordering, slot merging, op encoding, checkpoint
segments and the adjoint plan, for several tile shapes."""
import numpy as np
import pytest
import torch

from oracle import oracle
from qandle_gb300 import engine, workloads
from tests import program_emulator as emu


def _runtime(lo, desc, B):
    scales = lo.param_scale if len(lo.param_scale) == len(lo.param_mods) else [1.0] * len(lo.param_mods)
    params = np.array([sc * float(m.remapping(m.theta).reshape(-1)[0].detach())
                       for m, sc in zip(lo.param_mods, scales)])
    inputs = desc.get("inputs", {})
    cols = []
    for c, (name, j) in enumerate(lo.named_cols):
        v = np.asarray(inputs[name], dtype=np.float32).astype(np.float64)
        v = v[..., j] if j is not None else v
        if c < len(lo.named_scale):
            v = v * lo.named_scale[c]
        cols.append(np.broadcast_to(v, (B,)))
    named = np.stack(cols, 1) if cols else np.zeros((B, 1))
    umats = [np.asarray(u.numpy(), dtype=complex) for u in lo.umats]
    embed = None
    emb = [g for g in lo.gates if g[0] == 7]
    if emb:
        g = emb[-1]
        axis, k, col0, qoff = g[1], g[2], g[4], g[5]
        embed = np.zeros((B, lo.n, 2), complex)
        embed[:, :, 0] = 1.0
        for jj in range(k):
            q = lo.qlist[qoff + jj]
            m = np.stack([emu.row_matrix(axis, x) for x in named[:, col0 + jj]])
            v0, v1 = embed[:, q, 0].copy(), embed[:, q, 1].copy()
            embed[:, q, 0] = m[:, 0, 0] * v0 + m[:, 1, 0] * v1
            embed[:, q, 1] = m[:, 0, 1] * v0 + m[:, 1, 1] * v1
    return params, named, umats, embed


CASES = [
    ("sel_n10", lambda: workloads.sel_reupload(n=10, batch=3, layers=3, reupload_every=2, measure="z")),
    ("sel_n15", lambda: workloads.sel_reupload(n=15, batch=2, layers=3, reupload_every=2, measure="z")),
    ("brick_n14", lambda: workloads.adjoint_brick(n=14, batch=2, layers=4)),
    ("deep_n14", lambda: workloads.deep_u(n=14, batch=1, layers=4)),
    ("plain_n8", lambda: workloads.plain_small(n=8, batch=5, layers=2)),
]
OPTS = [dict(tile_bits=13, low_bits=6, max_high=0), dict(tile_bits=12, low_bits=4, max_high=2),
        dict(tile_bits=11, low_bits=5, max_high=1), dict(tile_bits=13, low_bits=8, max_high=3),
        dict(tile_bits=13, low_bits=6, reg_bits=4), dict(tile_bits=12, low_bits=5, reg_bits=4),
        dict(tile_bits=13, low_bits=6, reg_search=1), dict(tile_bits=13, low_bits=6, max_high=4, reg_search=1),
        dict(tile_bits=13, low_bits=6, fwd_max_mats=3), dict(tile_bits=12, low_bits=5, fwd_max_mats=1 << 30)]


@pytest.mark.parametrize("case", [c[0] for c in CASES])
@pytest.mark.parametrize("oi", range(len(OPTS)))
def test_forward_plan_matches_oracle(case, oi):
    desc = dict(CASES)[case]()
    desc["measure"] = "state"
    circ = workloads.build_circuit(desc, engine="fused")
    lo = engine.lower(circ.circuit)
    B = desc["batch"]
    prog = engine.Program(lo, "state", keep_state=True, segments=2, **OPTS[oi])
    params, named, umats, embed = _runtime(lo, desc, B)
    st, ck = emu.run_forward(prog, desc["n"], B, params, named, umats, embed=embed)
    ref = oracle.run(desc)
    assert np.abs(st - ref).max() < 1e-10
    assert prog.info.forward_passes >= 1


@pytest.mark.parametrize("rb,cap", [(5, 0), (4, 0), (5, 7)])
@pytest.mark.parametrize("case", ["sel_n10", "brick_n14", "deep_n14", "sel_n15"])
def test_backward_plan_matches_oracle(case, rb, cap):
    desc = dict(CASES)[case]()
    desc["measure"] = "p0"
    n, B = desc["n"], desc["batch"]
    circ = workloads.build_circuit(desc, engine="fused")
    lo = engine.lower(circ.circuit)
    prog = engine.Program(lo, "p0", keep_state=True, segments=3, tile_bits=13, low_bits=5, reg_bits=rb,
                          bwd_max_grad=cap)
    params, named, umats, embed = _runtime(lo, desc, B)
    st, ck = emu.run_forward(prog, n, B, params, named, umats, embed=embed)
    w = np.linspace(-1.0, 1.0, B * n).reshape(B, n)
    # lambda = dL/dpsi* for L = sum(w * P0)
    amp = np.arange(1 << n)
    wt = np.zeros((B, 1 << n))
    for q in range(n):
        wt += np.where(((amp >> (n - 1 - q)) & 1) == 0, 1.0, 0.0)[None, :] * w[:, q:q + 1]
    lam = wt * st
    tg = prog.grad_targets()
    dp, dn, _ = emu.run_backward(prog, n, B, params, named, umats, st, lam, ck, tg)
    rdp, rdn, _ = oracle.adjoint(desc, w, "p0")
    assert dp.size == rdp.size and (dp.size == 0 or np.abs(dp - rdp).max() < 1e-9)
    # every occurrence of a named input has its own column; sum them per
    # input the way autograd does, then compare with the oracle's totals
    got = {}
    for c, (name, j) in enumerate(lo.named_cols):
        ref = rdn[name]
        arr = got.setdefault(name, np.zeros_like(ref))
        if j is None:
            arr += dn[:, c] if arr.ndim == 1 else dn[:, c:c + 1]
        else:
            arr[:, j] += dn[:, c]
    for name, arr in got.items():
        assert np.abs(arr - rdn[name]).max() < 1e-9, name


def test_backward_rotation_cap_splits_passes():
    """bwd_max_grad caps the gradient-carrying rotations of every backward
    pass (default 28; at most the kernel's shared-memory limit, 64 at 16
    amplitudes per thread); a lower cap gives more, shorter passes."""
    desc = workloads.adjoint_brick(n=16, batch=1, layers=20)
    circ = workloads.build_circuit(desc, engine="fused")
    lo = engine.lower(circ.circuit)
    full = engine.Program(lo, "p0", keep_state=True, segments=4, bwd_max_grad=100)  # the 64 limit
    capped = engine.Program(lo, "p0", keep_state=True, segments=4, bwd_max_grad=32)
    default = engine.Program(lo, "p0", keep_state=True, segments=4)
    assert max(p["ngrad"] for p in default.passes(backward=True)) <= 28
    assert max(p["ngrad"] for p in full.passes(backward=True)) == 64

    assert max(p["ngrad"] for p in capped.passes(backward=True)) <= 32
    assert max(p["ngrad"] for p in full.passes(backward=True)) <= 64
    assert capped.info.backward_passes > full.info.backward_passes
    assert sum(p["ngrad"] for p in capped.passes(backward=True)) == sum(p["ngrad"] for p in full.passes(backward=True))
    with pytest.raises(RuntimeError):
        engine.Program(lo, "p0", keep_state=True, bwd_max_grad=-1)


def test_forward_mat_cap():
    """A forward pass holds at most 24 2x2 slots by default (fwd_max_mats):
    a 13-qubit, 20-layer SEL circuit that fits one pass uncapped is split,
    with the same gates in the same order."""
    desc = workloads.sel_reupload(n=13, batch=2, layers=20)
    circ = workloads.build_circuit(desc, engine="fused")
    lo = engine.lower(circ.circuit)

    def mats(prog):
        return [int(np.sum((p["ops"][:, 0] == 2) | (p["ops"][:, 0] == 3))) for p in prog.passes()]

    default = engine.Program(lo, "z", keep_state=False)
    uncapped = engine.Program(lo, "z", keep_state=False, fwd_max_mats=1 << 30)
    assert uncapped.info.forward_passes == 1 and max(mats(uncapped)) > 24
    assert max(mats(default)) <= 24 and default.info.forward_passes > 1
    assert sum(mats(default)) == sum(mats(uncapped))
    assert max(mats(engine.Program(lo, "z", keep_state=False, fwd_max_mats=10))) <= 10
    with pytest.raises(RuntimeError):
        engine.Program(lo, "z", keep_state=False, fwd_max_mats=-1)


def test_fusion_reduces_passes():
    desc = workloads.sel_reupload(n=20, batch=1, layers=10)
    circ = workloads.build_circuit(desc, engine="fused")
    lo = engine.lower(circ.circuit)
    prog = engine.Program(lo, "z", keep_state=False)
    gates = len(lo.gates)
    # every pass is one HBM round trip; the plain form needs one per gate
    assert prog.info.forward_passes * 10 <= gates, prog.summary()


def test_planner_rejects_bad_programs():
    from qandle_gb300 import _lib
    import ctypes

    lib = _lib.load()
    g = (_lib.Gate * 1)(_lib.Gate(0, 9, 0, 0, 0, 0))  # qubit 9 in a 6-qubit circuit
    h = ctypes.c_void_p()
    rc = lib.qg_program_create(g, 1, None, 6, None, ctypes.byref(h))
    assert rc == 1 and b"out of range" in lib.qg_last_error()
    rc = lib.qg_program_create(g, 1, None, 3, None, ctypes.byref(h))
    assert rc == 1 and b"num_qubits" in lib.qg_last_error()


def test_serving_lowering_matches_front_end():
    from qandle_gb300 import serve

    rng = np.random.default_rng(5)
    for _ in range(6):
        d = workloads.random_sel_request(rng, n_range=(5, 12), depth_range=(2, 5), batch_max=8)
        lo_s, params, named, shift = serve.lower_description(d)
        lo_f = engine.lower(workloads.build_circuit(d, engine="fused").circuit)
        assert shift == 0
        assert lo_s.gates == lo_f.gates and lo_s.qlist == lo_f.qlist
        assert lo_s.named_cols == lo_f.named_cols
        p_f = np.array([float(m.remapping(m.theta).reshape(-1)[0].detach()) for m in lo_f.param_mods])
        assert np.array_equal(params[:len(p_f)], p_f.astype(np.float32))
    # narrow circuits get an idle qubit 0 and keep their results
    d = workloads.random_sel_request(rng, n_range=(4, 4), depth_range=(2, 3), batch_max=4)
    lo_s, params, named, shift = serve.lower_description(d)
    assert shift == 1 and lo_s.n == 5
    prog = engine.Program(lo_s, "state", keep_state=True)
    B = d["batch"]
    embed = np.zeros((B, 5, 2), complex)
    embed[:, :, 0] = 1.0
    for j in range(4):
        m = np.stack([emu.row_matrix(0, x) for x in named[:, j]])
        embed[:, j + 1, 0], embed[:, j + 1, 1] = m[:, 0, 0], m[:, 0, 1]
    st, _ = emu.run_forward(prog, 5, B, params.astype(np.float64), named.astype(np.float64), [], embed=embed)
    z = 2 * oracle.measure_p0(st) - (np.abs(st) ** 2).sum(-1, keepdims=True)
    d2 = dict(d)
    d2["measure"] = "z"
    assert np.abs(z[:, 1:] - oracle.forward(d2)).max() < 1e-9


def test_controlled_and_inverted_gates_plan_matches_oracle():
    """Controlled rotations (decomposed into rotations and CNOTs), named
    controlled rotations and inverted gates: planned, emulated, and equal to
    the oracle's controlled / inverse kinds (forward and adjoint)."""
    from tests import test_special_gpu as sp

    layers, desc, inputs = sp._mixed(n=9, batch=2, seed=8)
    n, B = desc["n"], desc["batch"]
    import qandle_gb300 as q

    circ = q.Circuit(layers, num_qubits=n)
    lo = engine.lower(circ.circuit)
    prog = engine.Program(lo, "p0", keep_state=True, segments=2, tile_bits=13, low_bits=5)
    params, named, umats, embed = _runtime(lo, desc, B)
    st0 = np.zeros((B, 1 << n), complex)
    st0[:, 0] = 1
    st, ck = emu.run_forward(prog, n, B, params, named, umats, embed=embed, state=st0)
    ref = oracle.run(desc, state=st0)
    # controlled RX goes through H on the target, a complex64 matrix
    # (1/sqrt(2) to float precision): agreement is at 1e-8, not 1e-10
    assert np.abs(st - ref).max() < 1e-6


def _random_mix(seed: int, n: int = 14, ngates: int = 160) -> dict:
    """Random circuit dense in RX / RZ / RY and CNOT / CZ on few qubits, so
    that diagonal gates are held across CNOT controls and targets, across
    phases and across passes."""
    rng = np.random.default_rng(seed)
    gates = []
    for _ in range(ngates):
        r = rng.random()
        if r < 0.55:
            axis = ("rx", "ry", "rz")[rng.integers(3)]
            gates.append((axis, int(rng.integers(n)), float(rng.uniform(-3, 3)), None))
        else:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            gates.append(("cnot", a, b) if r < 0.85 else ("cz", a, b))
    return {"name": "mix", "n": n, "batch": 2, "gates": gates, "inputs": {}, "measure": "state",
            "targets": None}


@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("oi", [0, 1, 2, 4, 8, 9])
def test_held_diagonals_random_circuits_match_oracle(seed, oi):
    desc = _random_mix(seed)
    circ = workloads.build_circuit(desc, engine="fused")
    lo = engine.lower(circ.circuit)
    prog = engine.Program(lo, "state", keep_state=False, **OPTS[oi])
    params, named, umats, embed = _runtime(lo, desc, 2)
    st, _ = emu.run_forward(prog, desc["n"], 2, params, named, umats, embed=embed)
    assert np.abs(st - oracle.run(desc)).max() < 1e-10


@pytest.mark.parametrize("opts", [dict(tile_bits=13, low_bits=6), dict(tile_bits=11, low_bits=4, max_high=2),
                                  dict(tile_bits=13, low_bits=6, fwd_max_mats=5)])
def test_random_circuits_plan_matches_reference(opts):
    """The reference's output states for 30 random circuits over every gate
    kind of the path (tests/golden/random_circuits.npz): the front-end
    circuit, lowered, planned and emulated as the fused engine runs it,
    gives them for every circuit of 5 qubits or more."""
    from tests import golden_io
    from tests.golden import make_golden as mg

    z = golden_io.load("random_circuits")
    ran = 0
    for name, (desc, psi) in mg.random_circuit_descs().items():
        n, B = desc["n"], desc["batch"]
        if n < 5:
            continue
        lo = engine.lower(workloads.build_circuit(desc).circuit)
        prog = engine.Program(lo, "state", keep_state=False, **opts)
        params, named, umats, embed = _runtime(lo, desc, B)
        st, _ = emu.run_forward(prog, n, B, params, named, umats, state=psi.astype(complex), embed=embed)
        assert np.abs(st - z[f"{name}_out"]).max() < 2e-6, name
        ran += 1
    assert ran >= 15


@pytest.mark.parametrize("rb,cap", [(5, 0), (4, 0), (4, 3)])
def test_random_circuits_backward_plan_matches_reference_autograd(rb, cap):
    """The adjoint plan, emulated, gives torch autograd's gradients through
    the reference (tests/golden/random_grads.npz: loss sum(W * joint
    probabilities)) for the random circuits of 5 qubits or more, with a
    checkpoint in the middle."""
    from tests import golden_io
    from tests.golden import make_golden as mg

    z = golden_io.load("random_grads")
    ran = 0
    for name, (desc, psi) in mg.random_circuit_descs().items():
        if f"{name}_w" not in z.files or desc["n"] < 5:
            continue
        d = dict(desc, measure="probs")
        n, B = d["n"], d["batch"]
        lo = engine.lower(workloads.build_circuit(d).circuit)
        prog = engine.Program(lo, "probs", keep_state=True, segments=2, tile_bits=13, low_bits=5, reg_bits=rb,
                              bwd_max_grad=cap)
        params, named, umats, embed = _runtime(lo, d, B)
        st, ck = emu.run_forward(prog, n, B, params, named, umats, state=psi.astype(complex), embed=embed)
        lam = z[f"{name}_w"].astype(np.float64) * st  # dL/dpsi* for L = sum(W |psi|^2)
        dp, dn, _ = emu.run_backward(prog, n, B, params, named, umats, st, lam, ck, prog.grad_targets())
        assert np.abs(dp - z[f"{name}_dtheta"]).max() < 1e-5, name
        got = {}
        for c, (nm, j) in enumerate(lo.named_cols):
            got[nm] = got.get(nm, 0) + dn[:, c]
        for nm, v in got.items():
            assert np.abs(v - z[f"{name}_dnamed_{nm}"]).max() < 1e-5, (name, nm)
        ran += 1
    assert ran >= 5


@pytest.mark.timeout(120)
@pytest.mark.parametrize("training", [False, True])
def test_long_low_run_leaves_room_for_two_qubit_gates(training):
    """With low_bits = tile_bits - 1 a two-qubit gate between two strided
    qubits does not fit a tile of one strided slot.  The planner keeps at
    least two strided slots (the forward and the narrower backward tiles),
    so such options plan in bounded time and give the oracle's state (this
    case used to loop in the planner)."""
    rng = np.random.default_rng(11)
    n = 14
    gates = []
    for _ in range(40):
        if rng.random() < 0.5:
            gates.append((("rx", "ry", "rz")[rng.integers(3)], int(rng.integers(n)), float(rng.uniform(-3, 3)), None))
        else:
            a, b = (int(x) for x in rng.choice(3, 2, replace=False))  # qubits 0..2: the strided bits
            gates.append(("cnot", a, b))
    desc = {"name": "mix", "n": n, "batch": 2, "gates": gates, "inputs": {}, "measure": "state", "targets": None}
    lo = engine.lower(workloads.build_circuit(desc, engine="fused").circuit)
    prog = engine.Program(lo, "state", keep_state=training, segments=2 if training else 1,
                          tile_bits=12, low_bits=11, max_high=1)
    params, named, umats, embed = _runtime(lo, desc, 2)
    st, _ = emu.run_forward(prog, n, 2, params, named, umats, embed=embed)
    assert np.abs(st - oracle.run(desc)).max() < 1e-10


def test_executor_picks_uncapped_plan_for_calls_that_do_not_fill_the_gpu(monkeypatch):
    """FusedExecutor.program(training, batch, device): with the default pass
    length, a call whose passes have fewer tiles than the device has SMs
    gets the uncapped plan (one pass for this 13-qubit circuit), a larger
    call the capped plan; without a batch, the plan the last call used.  An
    explicit fwd_max_mats is always kept."""
    import torch

    monkeypatch.setattr(engine, "_sm_count", lambda dev: 152)
    desc = workloads.sel_reupload(n=13, batch=2, layers=12, reupload_every=4)
    circ = workloads.build_circuit(desc, engine="fused")
    ex = engine.FusedExecutor(circ.circuit)
    dev = torch.device("cuda", 0)
    small = ex.program(False, 4, dev)        # 4 tiles
    assert small.info.forward_passes == 1
    assert ex.program(False) is small        # the last call's plan
    large = ex.program(False, 304, dev)      # 304 tiles
    assert large.info.forward_passes > 1
    assert ex.program(False) is large
    fixed = engine.FusedExecutor(circ.circuit, fwd_max_mats=10)
    assert fixed.program(False, 4, dev).info.forward_passes > 1

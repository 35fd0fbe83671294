"""Generate the golden vectors in tests/golden/ by running the reference itself.

Run in a container that has the reference sources (qandle 0.1.8, pure Python
on torch):

    python tests/golden/make_golden.py --reference /path/to/qandle/src

qandle imports the third-party ``qw_map`` package (qw-map 0.1.2), which is not
installed here; every parity case uses ``remapping=None``, which qandle maps
to ``qw_map.none`` (the identity, operators.py:168-170), so a stand-in module
with ``none`` = identity is placed on the path.  Its ``tanh`` raises, so a case
that would silently use the unpinned default mapping fails instead.

The cases follow the reference's own tests with the reference in PennyLane's
place (PennyLane is not installed): per-gate sweeps
(test/test_operators.py:85-128, :157-203), re-uploading (:131-154),
embeddings (test/test_embeddings.py:56-153), measurements
(test/test_measurements.py:6-48), strongly entangling layers
(test/test_ansaetze.py:6-83), plus small instances of the four measured
circuit families and torch-autograd gradients through the reference; the
special gates (Invert, Controlled, Reset), AmplitudeEmbedding, the OpenQASM
export, the splitter's subcircuits, the other ansaetze and the to_matrix()
results of gates, ansaetze and circuits.

Output: one compressed .npz per group, arrays only (no pickles).  Circuit
descriptions are stored as JSON strings next to their arrays.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from qandle_gb300 import workloads  # noqa: E402

QW_STUB = '''
def none(x):
    return x


def tanh(x):
    raise RuntimeError("qw_map.tanh is not pinned for parity; use remapping=None")
'''


def import_reference(src: str):
    stub = tempfile.mkdtemp(prefix="qwstub")
    os.makedirs(os.path.join(stub, "qw_map"))
    with open(os.path.join(stub, "qw_map", "__init__.py"), "w") as f:
        f.write(QW_STUB)
    sys.path.insert(0, stub)
    sys.path.insert(0, src)
    import qandle  # noqa: F401

    return qandle


def desc_json(desc: dict) -> str:
    gates = []
    for g in desc["gates"]:
        if g[0] == "u":
            m = np.asarray(g[2], dtype=np.complex64)
            gates.append(["u", g[1], [[float(v.real), float(v.imag)] for v in m.reshape(-1)]])
        else:
            gates.append(list(g))
    d = {k: v for k, v in desc.items() if k not in ("gates", "inputs", "targets")}
    d["gates"] = gates
    d["input_names"] = sorted(desc.get("inputs", {}).keys())
    return json.dumps(d)


def to_reference(qandle, desc: dict, thetas_require_grad: bool = False):
    layers, params = [], []
    for g in desc["gates"]:
        k = g[0]
        if k == "emb":
            layers.append(qandle.AngleEmbedding(name=g[2], qubits=list(g[3]), rotation=g[1]))
        elif k in ("rx", "ry", "rz"):
            cls = {"rx": qandle.RX, "ry": qandle.RY, "rz": qandle.RZ}[k]
            if g[3] is None:
                th = torch.tensor(np.float32(g[2]), dtype=torch.float, requires_grad=True)
                params.append(th)
                layers.append(cls(qubit=g[1], theta=th, remapping=None))
            else:
                layers.append(cls(qubit=g[1], name=g[3], remapping=None))
        elif k == "u":
            layers.append(qandle.U(qubit=g[1], matrix=torch.tensor(np.asarray(g[2], np.complex64))))
        elif k == "cnot":
            layers.append(qandle.CNOT(control=g[1], target=g[2]))
        elif k == "cz":
            layers.append(qandle.CZ(control=g[1], target=g[2]))
        elif k == "swap":
            layers.append(qandle.SWAP(a=g[1], b=g[2]))
    m = desc.get("measure")
    if m == "probs":
        layers.append(qandle.MeasureJointProbability())
    elif m in ("p0", "z"):
        layers.append(qandle.MeasureProbability())
    circ = qandle.Circuit(layers, num_qubits=desc["n"])
    return circ


def ref_thetas(qandle, circ):
    """Theta parameters of the built reference circuit in gate order."""
    out = []
    for mod in circ.circuit.layers:
        if isinstance(mod, qandle.operators.BuiltParametrizedOperator) and not mod.named:
            out.append(mod.theta)
    return out


def kwargs_of(desc: dict, requires_grad: bool = False):
    kw = {}
    for k, v in desc.get("inputs", {}).items():
        t = torch.tensor(np.asarray(v, dtype=np.float32))
        kw[k] = t
    return kw


def gate_cases(qandle):
    """Per-gate sweeps, as test_operators.py:85-128 (unbatched, theta=0.543321)
    and :157-203 (batch 13, theta=-2.3456), plus U with non-symmetric
    matrices so the row-vector convention is pinned."""
    out = {}
    idx = 0
    for batched, v in ((False, 0.543321), (True, -2.3456)):
        torch.manual_seed(42)
        for n in range(1, 6):
            inp = torch.rand(13, 2 ** n, dtype=torch.cfloat) if batched else \
                torch.rand(2 ** n, dtype=torch.cfloat)
            inp = inp / torch.linalg.norm(inp, dim=-1, keepdim=True)
            for w in range(n):
                specs = [("rx", w), ("ry", w), ("rz", w)]
                specs += [(k, w, w2) for w2 in range(n) if w2 != w for k in ("cnot", "cz", "swap")]
                for sp in specs:
                    if sp[0] in ("rx", "ry", "rz"):
                        cls = {"rx": qandle.RX, "ry": qandle.RY, "rz": qandle.RZ}[sp[0]]
                        op = cls(qubit=w, theta=v, remapping=None).build(num_qubits=n)
                        gate = [sp[0], w, float(np.float32(v)), None]
                    else:
                        cls = {"cnot": qandle.CNOT, "cz": qandle.CZ, "swap": qandle.SWAP}[sp[0]]
                        op = (cls(sp[1], sp[2]) if sp[0] != "swap" else cls(a=sp[1], b=sp[2]))
                        op = op.build(num_qubits=n)
                        gate = list(sp)
                    res = op(inp).detach()
                    out[f"g{idx}_in"] = inp.numpy()
                    out[f"g{idx}_out"] = res.numpy()
                    out[f"g{idx}_desc"] = np.array(json.dumps({"n": n, "gate": gate}))
                    idx += 1
    # U with random non-symmetric complex matrices (U is not unitary-checked
    # by the reference; use unitary ones anyway)
    gen = torch.Generator().manual_seed(7)
    for n in range(1, 5):
        inp = torch.rand(5, 2 ** n, dtype=torch.cfloat, generator=gen)
        inp = inp / torch.linalg.norm(inp, dim=-1, keepdim=True)
        for w in range(n):
            a, b, c = (torch.rand(3, generator=gen) * 2 * np.pi).tolist()
            m = workloads.u3_row_matrix(a, b, c)
            op = qandle.U(qubit=w, matrix=torch.tensor(m)).build(num_qubits=n)
            res = op(inp).detach()
            out[f"g{idx}_in"] = inp.numpy()
            out[f"g{idx}_out"] = res.numpy()
            g = ["u", w, [[float(z.real), float(z.imag)] for z in m.reshape(-1)]]
            out[f"g{idx}_desc"] = np.array(json.dumps({"n": n, "gate": g}))
            idx += 1
    out["count"] = np.array(idx)
    return out


def random_circuit_descs() -> dict:
    """name -> description of random circuits over every gate kind of the
    path (fixed and named rotations, U, CNOT, CZ, SWAP) on 3..8 qubits, batch
    3, state output, and the seeded input state [3, 2^n]."""
    out = {}
    for seed in range(30):
        rng = np.random.default_rng(3000 + seed)
        n = int(rng.integers(3, 9))
        B = 3
        gates, inputs = [], {}
        for i in range(int(rng.integers(10, 60))):
            kind = ("rx", "ry", "rz", "u", "cnot", "cz", "swap")[int(rng.integers(7))]
            if kind in ("rx", "ry", "rz"):
                q = int(rng.integers(n))
                if rng.random() < 0.2:
                    name = f"a{i}"
                    inputs[name] = rng.uniform(-3, 3, size=B).astype(np.float32)
                    gates.append((kind, q, None, name))
                else:
                    gates.append((kind, q, float(np.float32(rng.uniform(-3, 3))), None))
            elif kind == "u":
                a, b, c = (float(v) for v in rng.uniform(0, 2 * np.pi, 3))
                gates.append(("u", int(rng.integers(n)), workloads.u3_row_matrix(a, b, c).astype(np.complex64)))
            else:
                a, b = (int(x) for x in rng.choice(n, 2, replace=False))
                gates.append((kind, a, b))
        psi = rng.normal(size=(B, 1 << n)) + 1j * rng.normal(size=(B, 1 << n))
        psi = (psi / np.linalg.norm(psi, axis=1, keepdims=True)).astype(np.complex64)
        out[f"rand{seed}"] = ({"n": n, "batch": B, "gates": gates, "inputs": inputs, "measure": "state"}, psi)
    return out


def random_circuit_cases(qandle):
    """The reference's output states for random_circuit_descs()."""
    out = {}
    for name, (desc, psi) in random_circuit_descs().items():
        circ = to_reference(qandle, desc)
        with torch.no_grad():
            st = circ(torch.tensor(psi), **kwargs_of(desc))
        out[f"{name}_out"] = st.numpy()
    return out


def random_grad_cases(qandle):
    """torch-autograd gradients of the reference for the first 12 random
    circuits with joint probabilities out and loss sum(W * probs), W seeded
    [3, 2^n]: d loss / d theta of the unnamed rotations (gate order) and
    d loss / d named input."""
    out = {}
    for i, (name, (desc, psi)) in enumerate(random_circuit_descs().items()):
        if i >= 12:
            break
        d = dict(desc, measure="probs")
        circ = to_reference(qandle, d)
        kw = {k: v.clone().requires_grad_(True) for k, v in kwargs_of(d).items()}
        w = torch.tensor(np.random.default_rng(4000 + i).uniform(-1, 1, size=(d["batch"], 1 << d["n"])),
                         dtype=torch.float32)
        probs = circ(torch.tensor(psi), **kw)
        (probs * w).sum().backward()
        thetas = ref_thetas(qandle, circ)
        out[f"{name}_w"] = w.numpy()
        out[f"{name}_dtheta"] = np.array([float(t.grad) if t.grad is not None else 0.0 for t in thetas],
                                         dtype=np.float64)
        for k, v in kw.items():
            out[f"{name}_dnamed_{k}"] = v.grad.numpy()
    return out


def embedding_cases(qandle):
    """test_embeddings.py:56-153 (x3, y4, z5, each unbatched and batched),
    plus a qubit subset and a repeated qubit."""
    out = {}
    torch.manual_seed(42)
    cases = [
        ("rx", 3, None, torch.arange(3).float() + 0.5),
        ("rx", 3, None, torch.rand(10, 3) + 0.5),
        ("ry", 4, None, torch.arange(4).float() + 2.5),
        ("ry", 4, None, torch.rand(10, 4) + 2.5),
        ("rz", 5, None, torch.arange(5).float() + 2.5),
        ("rz", 5, None, torch.rand(10, 5) + 2.5),
        ("rx", 4, [1, 3], torch.rand(6, 2) * 3.0),
        ("ry", 3, [0, 0, 2], torch.rand(6, 3) * 3.0),
    ]
    for i, (rot, n, qubits, x) in enumerate(cases):
        qs = list(range(n)) if qubits is None else qubits
        emb = qandle.AngleEmbedding(qubits=qs, rotation=rot, name="e").build(num_qubits=n)
        res = emb(e=x).detach()
        out[f"e{i}_x"] = x.numpy()
        out[f"e{i}_out"] = res.numpy()
        out[f"e{i}_desc"] = np.array(json.dumps({"n": n, "rot": rot, "qubits": qs}))
    out["count"] = np.array(len(cases))
    return out


def measurement_cases(qandle):
    """test_measurements.py:6-48 plus the squeeze quirks of
    measurements.py:120-123 (batch 1 and one qubit)."""
    out = {}
    torch.manual_seed(3)
    shapes = [(None, 3), (17, 3), (1, 3), (5, 1), (None, 1), (4, 6)]
    for i, (b, n) in enumerate(shapes):
        inp = torch.rand(2 ** n, dtype=torch.cfloat) if b is None else \
            torch.rand(b, 2 ** n, dtype=torch.cfloat)
        inp = inp / torch.linalg.norm(inp, dim=-1, keepdim=True)
        p0 = qandle.MeasureProbabilityBuilt(num_qubits=n)(inp).detach()
        pj = qandle.MeasureJointProbability()(inp).detach()
        out[f"m{i}_in"] = inp.numpy()
        out[f"m{i}_p0"] = p0.numpy()
        out[f"m{i}_joint"] = pj.numpy()
    out["count"] = np.array(len(shapes))
    return out


def sel_cases(qandle):
    """test_ansaetze.py:6-26 and :63-83 (remapping=None)."""
    out = {}
    torch.manual_seed(11)
    for i, (n, depth, batch) in enumerate(((4, 10, None), (5, 7, 17), (6, 3, 4))):
        inp = torch.rand(2 ** n, dtype=torch.cfloat) if batch is None else \
            torch.rand(batch, 2 ** n, dtype=torch.cfloat)
        inp = inp / torch.linalg.norm(inp, dim=-1, keepdim=True)
        w = torch.rand(depth, n, 3)
        sel = qandle.StronglyEntanglingLayer(qubits=list(range(n)), depth=depth, q_params=w,
                                             remapping=None).build(num_qubits=n)
        res = sel(inp).detach()
        out[f"s{i}_in"] = inp.numpy()
        out[f"s{i}_w"] = w.numpy()
        out[f"s{i}_out"] = res.numpy()
        out[f"s{i}_desc"] = np.array(json.dumps({"n": n, "depth": depth}))
    out["count"] = np.array(3)
    return out


def reupload_cases(qandle):
    """test_operators.py:131-154: a named RX equals the fixed-theta RX,
    unbatched, batched with a scalar input and with a [7] input."""
    q = 3
    v = torch.tensor(0.123)
    torch.manual_seed(42)
    c2 = qandle.Circuit(layers=[qandle.RX(qubit=1, name="reupload", remapping=None)],
                        num_qubits=q)
    inp_u = torch.rand(2 ** q, dtype=torch.cfloat)
    inp_u = inp_u / torch.linalg.norm(inp_u)
    inp_b = torch.rand(7, 2 ** q, dtype=torch.cfloat)
    inp_b = inp_b / torch.linalg.norm(inp_b, dim=-1, keepdim=True)
    vb = torch.rand(7) * 3.0
    return {
        "inp_u": inp_u.numpy(), "inp_b": inp_b.numpy(), "v": v.numpy(), "vb": vb.numpy(),
        "unb": c2(inp_u, reupload=v).detach().numpy(),
        "bat_scalar": c2(inp_b, reupload=v).detach().numpy(),
        "bat_vec": c2(inp_b, reupload=vb).detach().numpy(),
        "unb_vec": c2(inp_u, reupload=vb).detach().numpy(),
    }


def circuit_cases(qandle):
    """Small instances of the four measured families through qandle.Circuit,
    and torch-autograd gradients through the reference."""
    out = {}
    descs = {
        "plain_small": workloads.plain_small(),  # full size: 8 qubits, batch 64
        "sel_small": workloads.sel_reupload(n=6, batch=8, layers=4, reupload_every=2,
                                            measure="p0"),
        "brick_small": workloads.adjoint_brick(n=6, batch=8, layers=4),
        "deep_small": workloads.deep_u(n=6, batch=2, layers=6),
    }
    for name, desc in descs.items():
        circ = to_reference(qandle, desc)
        kw = kwargs_of(desc)
        if name == "deep_small":
            res = circ(torch.zeros(2, 2 ** 6, dtype=torch.cfloat).index_fill_(1, torch.tensor([0]), 1.0))
        else:
            res = circ(**kw) if kw else circ()
        out[f"{name}_desc"] = np.array(desc_json(desc))
        for k, v in desc.get("inputs", {}).items():
            out[f"{name}_in_{k}"] = np.asarray(v)
        out[f"{name}_out"] = res.detach().numpy()
    # gradients: brick_small with MSE(<Z>, targets), <Z> = 2 P0 - 1
    desc = descs["brick_small"]
    circ = to_reference(qandle, desc)
    circ.circuit.state = circ.circuit.state.expand(desc["batch"], -1).contiguous()
    p0 = circ()
    z = 2.0 * p0 - 1.0
    t = torch.tensor(desc["targets"])
    loss = ((z - t) ** 2).mean()
    loss.backward()
    ths = ref_thetas(qandle, circ)
    out["brick_small_targets"] = desc["targets"]
    out["brick_small_loss"] = np.array(loss.item())
    out["brick_small_dtheta"] = np.array([th.grad.item() for th in ths], dtype=np.float32)
    # gradients wrt the embedding inputs and shared thetas: sel_small, loss = sum(P0 * w)
    desc = descs["sel_small"]
    circ = to_reference(qandle, desc)
    kw = {k: v.clone().requires_grad_(True) for k, v in kwargs_of(desc).items()}
    # the re-uploads read columns of x; keep them tied to x for the gradient
    x = kw["x"]
    for q in range(desc["n"]):
        kw[f"up{q}"] = x[:, q]
    p0 = circ(**kw)
    wts = torch.linspace(-1.0, 1.0, p0.numel()).reshape(p0.shape)
    (p0 * wts).sum().backward()
    ths = ref_thetas(qandle, circ)
    out["sel_small_weights"] = wts.numpy()
    out["sel_small_dtheta"] = np.array([th.grad.item() for th in ths], dtype=np.float32)
    out["sel_small_dx"] = x.grad.numpy()
    return out


def special_cases(qandle):
    """Reset (test/test_operators.py:6-58 inputs), Invert of every gate kind,
    Controlled rotations and U (fixed and per-sample angles), the angle
    gradient through controlled rotations, and one circuit mixing them.
    Each case stores a JSON spec of how to build the op with the front end."""
    out = {}
    idx = 0

    def put(spec, inp, res, kw=None):
        nonlocal idx
        out[f"s{idx}_in"] = inp.detach().numpy()
        out[f"s{idx}_out"] = res.detach().numpy()
        out[f"s{idx}_spec"] = np.array(json.dumps(spec))
        if kw:
            for k, v in kw.items():
                out[f"s{idx}_kw_{k}"] = v.detach().numpy()
        idx += 1

    # Reset: the reference's own unbatched and batched inputs
    for batched in (False, True):
        torch.manual_seed(3)
        for n in range(1, 5):
            if batched:
                inp = torch.rand(7, 2 ** n, dtype=torch.cfloat)
                inp = inp / torch.linalg.norm(inp, dim=-1, keepdim=True)
            else:
                inp = torch.arange(2 ** n).to(torch.cfloat) + 0.5 - 0.1j
                inp = inp / torch.linalg.norm(inp)
            for q in range(n):
                op = qandle.Reset(qubit=q).build(num_qubits=n)
                put({"n": n, "op": "reset", "qubit": q}, inp, op(inp))
    gen = torch.Generator().manual_seed(11)
    # Invert of every gate kind
    for n in range(1, 5):
        inp = torch.rand(5, 2 ** n, dtype=torch.cfloat, generator=gen)
        inp = inp / torch.linalg.norm(inp, dim=-1, keepdim=True)
        for q in range(n):
            for k in ("rx", "ry", "rz"):
                th = float(np.float32(torch.rand(1, generator=gen).item() * 2 * np.pi))
                cls = {"rx": qandle.RX, "ry": qandle.RY, "rz": qandle.RZ}[k]
                tgt = cls(qubit=q, theta=th, remapping=None).build(num_qubits=n)
                op = qandle.Invert(tgt).build(num_qubits=n)
                put({"n": n, "op": "invert", "target": [k, q, th]}, inp, op(inp))
            a, b, c = (torch.rand(3, generator=gen) * 2 * np.pi).tolist()
            m = workloads.u3_row_matrix(a, b, c)
            tgt = qandle.U(qubit=q, matrix=torch.tensor(m)).build(num_qubits=n)
            op = qandle.Invert(tgt).build(num_qubits=n)
            put({"n": n, "op": "invert", "target": ["u", q, [[float(z.real), float(z.imag)] for z in m.reshape(-1)]]},
                inp, op(inp))
            for q2 in range(n):
                if q2 == q:
                    continue
                for k in ("cnot", "cz", "swap"):
                    cls = {"cnot": qandle.CNOT, "cz": qandle.CZ, "swap": qandle.SWAP}[k]
                    tgt = (cls(q, q2) if k != "swap" else cls(a=q, b=q2)).build(num_qubits=n)
                    op = qandle.Invert(tgt).build(num_qubits=n)
                    put({"n": n, "op": "invert", "target": [k, q, q2]}, inp, op(inp))
    # Controlled rotations and U
    for n in range(2, 5):
        inp = torch.rand(5, 2 ** n, dtype=torch.cfloat, generator=gen)
        inp = inp / torch.linalg.norm(inp, dim=-1, keepdim=True)
        for c in range(n):
            for t in range(n):
                if c == t:
                    continue
                for k in ("rx", "ry", "rz"):
                    th = float(np.float32(torch.rand(1, generator=gen).item() * 2 * np.pi))
                    cls = {"rx": qandle.RX, "ry": qandle.RY, "rz": qandle.RZ}[k]
                    op = qandle.Controlled(c, cls(qubit=t, theta=th, remapping=None)).build(num_qubits=n)
                    put({"n": n, "op": "controlled", "control": c, "target": [k, t, th]}, inp, op(inp))
                a, b, cc = (torch.rand(3, generator=gen) * 2 * np.pi).tolist()
                m = workloads.u3_row_matrix(a, b, cc)
                op = qandle.Controlled(c, qandle.U(qubit=t, matrix=torch.tensor(m))).build(num_qubits=n)
                put({"n": n, "op": "controlled", "control": c,
                     "target": ["u", t, [[float(z.real), float(z.imag)] for z in m.reshape(-1)]]}, inp, op(inp))
    # per-sample (named) controlled rotation
    n = 3
    inp = torch.rand(6, 2 ** n, dtype=torch.cfloat, generator=gen)
    inp = inp / torch.linalg.norm(inp, dim=-1, keepdim=True)
    x = torch.rand(6, generator=gen) * np.pi
    for k in ("rx", "ry", "rz"):
        cls = {"rx": qandle.RX, "ry": qandle.RY, "rz": qandle.RZ}[k]
        op = qandle.Controlled(2, cls(qubit=0, name="x", remapping=None)).build(num_qubits=n)
        put({"n": n, "op": "controlled", "control": 2, "target": [k, 0, None, "x"]}, inp, op(inp, x=x),
            kw={"x": x})
    # angle gradients through controlled rotations (autograd of the reference)
    n = 4
    inp = torch.rand(3, 2 ** n, dtype=torch.cfloat, generator=gen)
    inp = inp / torch.linalg.norm(inp, dim=-1, keepdim=True)
    ths = [torch.tensor(float(v), requires_grad=True) for v in (torch.rand(4, generator=gen) * 6).tolist()]
    layers = [qandle.RY(qubit=0, theta=ths[0], remapping=None), qandle.CNOT(0, 1),
              qandle.Controlled(1, qandle.RX(qubit=2, theta=ths[1], remapping=None)),
              qandle.Controlled(2, qandle.RY(qubit=3, theta=ths[2], remapping=None)),
              qandle.Controlled(3, qandle.RZ(qubit=0, theta=ths[3], remapping=None)),
              qandle.MeasureProbability()]
    circ = qandle.Circuit(layers, num_qubits=n)
    built_ths = [m.t.theta if hasattr(m, "t") and hasattr(m.t, "theta") else m.theta
                 for m in circ.circuit.layers if hasattr(m, "theta") or (hasattr(m, "t") and hasattr(m.t, "theta"))]
    p0 = circ(inp)
    loss = (p0 * torch.arange(1, p0.shape[-1] + 1)).sum()
    grads = torch.autograd.grad(loss, built_ths)
    out["grad_in"] = inp.numpy()
    out["grad_p0"] = p0.detach().numpy()
    out["grad_thetas"] = np.array([float(t.detach()) for t in built_ths], dtype=np.float32)
    out["grad_out"] = np.array([float(g) for g in grads], dtype=np.float64)
    # one circuit mixing the new gates with the usual ones, |psi|^2 out
    n = 6
    inp = torch.rand(4, 2 ** n, dtype=torch.cfloat, generator=gen)
    inp = inp / torch.linalg.norm(inp, dim=-1, keepdim=True)
    spec_layers, layers = [], []
    for d in range(2):
        for q in range(n):
            th = float(np.float32(torch.rand(1, generator=gen).item() * 6))
            layers.append(qandle.RY(qubit=q, theta=th, remapping=None))
            spec_layers.append(["ry", q, th])
        for q in range(n - 1):
            th = float(np.float32(torch.rand(1, generator=gen).item() * 6))
            layers.append(qandle.Controlled(q, qandle.RZ(qubit=q + 1, theta=th, remapping=None)))
            spec_layers.append(["controlled", q, ["rz", q + 1, th]])
        th = float(np.float32(torch.rand(1, generator=gen).item() * 6))
        tgt = qandle.RX(qubit=d, theta=th, remapping=None).build(num_qubits=n)
        layers.append(qandle.Invert(tgt))
        spec_layers.append(["invert", ["rx", d, th]])
        layers.append(qandle.CNOT(n - 1, 0))
        spec_layers.append(["cnot", n - 1, 0])
    layers.append(qandle.MeasureJointProbability())
    circ = qandle.Circuit(layers, num_qubits=n)
    put({"n": n, "op": "circuit", "layers": spec_layers, "measure": "probs"}, inp, circ(inp))
    out["count"] = np.array(idx)
    return out


def amplitude_cases(qandle):
    """AmplitudeEmbedding (embeddings.py:29-111) with and without padding and
    normalisation, its input gradient through a circuit, and QConv
    (convolution.py:9-61) with the SEL angles recorded (their remapping set
    to the identity: qandle's default remapping is qw_map.tanh, unpinned)."""
    out = {}
    gen = torch.Generator().manual_seed(21)
    idx = 0
    for n in range(1, 6):
        for length in sorted({2 ** n, max(1, 2 ** n - 3), 1}):
            for normalize in (False, True):
                pad = None if length == 2 ** n else 0.25
                x = torch.rand(4, length, generator=gen) + 0.1
                op = qandle.AmplitudeEmbedding(name="x", qubits=list(range(n)), normalize=normalize,
                                               pad_with=pad).build(num_qubits=n)
                res = op(x=x)
                out[f"a{idx}_x"] = x.numpy()
                out[f"a{idx}_out"] = res.detach().numpy()
                out[f"a{idx}_spec"] = np.array(json.dumps({"n": n, "normalize": normalize, "pad": pad}))
                idx += 1
    out["count"] = np.array(idx)
    # input gradient through an amplitude-embedded circuit
    n = 3
    x = (torch.rand(3, 6, generator=gen) + 0.1).requires_grad_(True)
    th = (torch.rand(n, generator=gen) * 6).tolist()
    layers = [qandle.AmplitudeEmbedding(name="x", qubits=list(range(n)), normalize=True, pad_with=0.0)]
    layers += [qandle.RY(qubit=q, theta=th[q], remapping=None) for q in range(n)]
    layers += [qandle.CNOT(0, 1), qandle.CNOT(1, 2), qandle.MeasureProbability()]
    circ = qandle.Circuit(layers, num_qubits=n)
    p0 = circ(x=x)
    (p0 * torch.arange(1, n + 1)).sum().backward()
    out["grad_x"] = x.detach().numpy()
    out["grad_th"] = np.array(th, dtype=np.float32)
    out["grad_p0"] = p0.detach().numpy()
    out["grad_dx"] = x.grad.numpy()
    # QConv: SEL angles recorded, remapping set to the identity
    for ci, (c_in, c_out, h, w, pad) in enumerate(((1, 3, 5, 6, 1), (2, 5, 4, 4, 0))):
        torch.manual_seed(100 + ci)
        conv = qandle.QConv(in_channels=c_in, out_channels=c_out, padding=pad)
        thetas = []
        for m in conv.qcircuit.circuit.layers[1].mods:
            if hasattr(m, "theta"):
                m.remapping = _qw_none
                thetas.append(float(m.theta.detach()))
        x = torch.rand(2, c_in, h, w, generator=gen)
        y = conv(x)
        out[f"qconv{ci}_x"] = x.numpy()
        out[f"qconv{ci}_thetas"] = np.array(thetas, dtype=np.float32)
        out[f"qconv{ci}_out"] = y.detach().numpy()
        out[f"qconv{ci}_cfg"] = np.array(json.dumps({"c_in": c_in, "c_out": c_out, "padding": pad}))
    return out


def amplitude_crop_cases(qandle):
    """AmplitudeEmbedding with more features than 2^n amplitudes and a
    pad value: the reference pads with a negative width, which torch's pad
    turns into cutting the features past 2^n (embeddings.py:50-62), then
    normalises what is left."""
    out = {}
    gen = torch.Generator().manual_seed(23)
    idx = 0
    for n, length in ((1, 3), (2, 7), (3, 9), (4, 20)):
        for normalize in (False, True):
            x = torch.rand(3, length, generator=gen) + 0.1
            op = qandle.AmplitudeEmbedding(name="x", qubits=list(range(n)), normalize=normalize,
                                           pad_with=0.5).build(num_qubits=n)
            out[f"c{idx}_x"] = x.numpy()
            out[f"c{idx}_out"] = op(x=x).detach().numpy()
            out[f"c{idx}_spec"] = np.array(json.dumps({"n": n, "normalize": normalize, "pad": 0.5}))
            idx += 1
    out["count"] = np.array(idx)
    return out


def qasm_circuits(qandle_mod):
    """Circuits whose OpenQASM export is compared as text (the random hash in
    embedding and measurement names is normalised)."""
    Q = qandle_mod
    return {
        "rot_fixed": ([Q.RX(0, theta=0.25, remapping=None), Q.RY(1, theta=-1.5, remapping=None),
                       Q.RZ(2, theta=3.0, remapping=None), Q.CNOT(0, 2), Q.CZ(1, 2),
                       Q.MeasureProbability()], 3),
        "named": ([Q.AngleEmbedding(name="x", qubits=[0, 1, 2], rotation="ry"), Q.RZ(1, name="up", remapping=None),
                   Q.CNOT(2, 0), Q.MeasureProbability()], 3),
        "special": ([Q.Reset(qubit=1), Q.Controlled(0, Q.RY(1, theta=0.5, remapping=None)),
                     Q.Invert(Q.RX(2, theta=0.75, remapping=None).build(num_qubits=3))], 3),
        "sel": ([Q.StronglyEntanglingLayer(qubits=[0, 1, 2], depth=2, remapping=None,
                                           q_params=torch.arange(18, dtype=torch.float32).reshape(2, 3, 3) / 10)],
                3),
        "twolocal": ([Q.TwoLocal(qubits=[0, 1, 2], depth=2, remapping=None, q_params=torch.full((2, 3), 0.3))], 3),
        "u_swap": ([Q.U(1, matrix=torch.tensor([[0.6, 0.8], [0.8, -0.6]], dtype=torch.cfloat)), Q.SWAP(0, 2),
                    Q.CNOT(0, 1)], 3),
        "nested": ([Q.Circuit([Q.RX(0, theta=0.1, remapping=None), Q.CNOT(0, 1)], num_qubits=3),
                    Q.RZ(2, theta=0.4, remapping=None)], 3),
    }


def qasm_cases(qandle):
    """OpenQASM 2 and 3 text of qasm_circuits() (the built TwoLocal's
    rotations take the default remapping, set to the identity here)."""
    import qandle.config as ref_config

    out = {}
    saved = ref_config.DEFAULT_MAPPING
    ref_config.DEFAULT_MAPPING = _qw_none
    try:
        for name, (layers, n) in qasm_circuits(qandle).items():
            circ = qandle.Circuit(layers, num_qubits=n)
            out[f"{name}_qasm2"] = np.array(circ.to_openqasm2())
            out[f"{name}_qasm3"] = np.array(circ.to_openqasm3())
    finally:
        ref_config.DEFAULT_MAPPING = saved
    return out


def split_layers(Q, gates):
    """Layers from ("cnot", c, t) / (axis, qubit, theta or None, name or None)."""
    out = []
    for g in gates:
        if g[0] == "cnot":
            out.append(Q.CNOT(g[1], g[2]))
        else:
            cls = {"rx": Q.RX, "ry": Q.RY, "rz": Q.RZ}[g[0]]
            kw = {}
            if g[2] is not None:
                kw["theta"] = float(g[2])
            if g[3] is not None:
                kw["name"] = g[3]
            out.append(cls(g[1], **kw))
    return out


def split_record(circuit) -> list:
    """Subcircuits of a split Circuit as plain data: mapping and gates
    (("cnot", c, t) / (axis, qubit, theta or None, name or None)), no
    remapping evaluated."""
    out = []
    for sc in circuit.circuit.subcircuits:
        layers = []
        for la in sc.layers:
            kind = type(la).__name__.replace("Built", "").lower()
            if kind == "cnot":
                layers.append(["cnot", int(la.c), int(la.t)])
            else:
                th = None if la.named else float(la.theta.detach().reshape(-1)[0])
                layers.append([kind, int(la.qubit), th, la.name])
        out.append({"mapping": sorted([int(k), int(v)] for k, v in sc.mapping.items()), "layers": layers})
    return out


def split_circuits() -> dict:
    """name -> (gates, num_qubits, max_qubits, via) for the splitter fixtures;
    via "method" is Circuit(...).split(k), "constructor" is
    Circuit(..., split_max_qubits=k)."""
    cnot10 = [("cnot", 0, 1), ("cnot", 0, 2), ("cnot", 1, 2), ("cnot", 2, 3), ("cnot", 3, 4), ("cnot", 4, 3),
              ("cnot", 3, 4), ("cnot", 4, 3), ("cnot", 3, 4), ("cnot", 4, 3), ("cnot", 3, 4), ("cnot", 4, 3),
              ("cnot", 3, 5), ("cnot", 5, 6), ("cnot", 6, 7), ("cnot", 6, 1), ("cnot", 7, 8), ("cnot", 8, 9)]
    cases = {
        "cnot10_k5": (cnot10, 10, 5, "method"),
        "cnot10_k3": (cnot10, 10, 3, "method"),
        "dummy_k2": ([("rx", 0, 0.3, None), ("cnot", 0, 2), ("ry", 1, -0.7, None), ("cnot", 1, 2)], 3, 2,
                     "constructor"),
    }
    sel = []
    for d, rng in enumerate((1, 2)):
        for q in range(6):
            for r, axis in enumerate(("rz", "ry", "rz")):
                sel.append((axis, q, round(0.1 * (1 + q + 6 * r + 18 * d), 4), None))
        for q in range(6):
            sel.append(("cnot", q, (q + rng) % 6))
    cases["sel6_k3"] = (sel, 6, 3, "method")
    cases["sel6_k4"] = (sel, 6, 4, "constructor")
    for seed in range(6):
        rng = np.random.default_rng(100 + seed)
        n = int(rng.integers(5, 9))
        gates = [("cnot", q, q + 1) for q in range(n - 1)]  # every qubit meets a CNOT
        for _ in range(int(rng.integers(30, 70))):
            if rng.random() < 0.5:
                a, b = (int(x) for x in rng.choice(n, 2, replace=False))
                gates.append(("cnot", a, b))
            else:
                axis = ("rx", "ry", "rz")[int(rng.integers(3))]
                q = int(rng.integers(n))
                if rng.random() < 0.15:
                    gates.append((axis, q, None, f"in{q}"))
                else:
                    gates.append((axis, q, round(float(rng.uniform(-3, 3)), 4), None))
        perm = rng.permutation(len(gates))
        gates = [gates[i] for i in perm]
        k = int(rng.integers(2, 6))
        cases[f"random{seed}_k{k}"] = (gates, n, k, "method" if seed % 2 == 0 else "constructor")
    # a wider random sweep: 3..8 qubits, 5..60 gates, any k >= 2 that splits
    for seed in range(40):
        rng = np.random.default_rng(2000 + seed)
        n = int(rng.integers(3, 9))
        gates = [("cnot", q, q + 1) for q in range(n - 1)]
        for _ in range(int(rng.integers(5, 60))):
            if rng.random() < 0.5:
                a, b = (int(x) for x in rng.choice(n, 2, replace=False))
                gates.append(("cnot", a, b))
            else:
                axis = ("rx", "ry", "rz")[int(rng.integers(3))]
                gates.append((axis, int(rng.integers(n)), round(float(rng.uniform(-3, 3)), 4), None))
        perm = rng.permutation(len(gates))
        gates = [gates[i] for i in perm]
        k = int(rng.integers(2, n))
        cases[f"sweep{seed}_k{k}"] = (gates, n, k, "method" if seed % 2 else "constructor")
    return cases


def build_split(Q, gates, n, k, via):
    layers = split_layers(Q, gates)
    if via == "constructor":
        return Q.Circuit(layers=layers, num_qubits=n, split_max_qubits=k)
    return Q.Circuit(layers=layers, num_qubits=n).split(max_qubits=k)


def split_inputs(n: int, gates) -> tuple:
    """Seeded input state [2^n] (complex128, normalised) and named inputs
    (name -> float) for running a split circuit."""
    rng = np.random.default_rng(7)
    psi = rng.normal(size=(1 << n,)) + 1j * rng.normal(size=(1 << n,))
    psi /= np.linalg.norm(psi)
    names = sorted({g[3] for g in gates if g[0] != "cnot" and g[3] is not None})
    return psi, {nm: 0.25 + 0.1 * i for i, nm in enumerate(names)}


def splitter_cases(qandle):
    """The reference splitter's subcircuits (qandle/splitter/main.py) for the
    circuits of split_circuits(), as JSON, and the split circuit's output state
    for split_inputs().  The splitter gives its rotations the default
    remapping (qw_map.tanh, unpinned), so the states are made with the
    identity as default remapping."""
    import qandle.config as ref_config

    out = {}
    saved = ref_config.DEFAULT_MAPPING
    ref_config.DEFAULT_MAPPING = _qw_none
    try:
        for name, (gates, n, k, via) in split_circuits().items():
            circ = build_split(qandle, gates, n, k, via)
            out[name] = np.array(json.dumps(split_record(circ)))
            psi, named = split_inputs(n, gates)
            with torch.no_grad():
                st = circ(torch.tensor(psi, dtype=torch.cfloat),
                          **{nm: torch.tensor(v, dtype=torch.float32) for nm, v in named.items()})
            out[name + "_state"] = st.numpy().astype(np.complex128)
    finally:
        ref_config.DEFAULT_MAPPING = saved
    return out


def ansatz_circuits() -> dict:
    """name -> (kind, num_qubits, constructor arguments) for the ansatz fixtures."""
    return {
        "twolocal_full": ("twolocal", 4, dict(qubits=[0, 1, 2, 3], depth=3)),
        "twolocal_sub": ("twolocal", 4, dict(qubits=[1, 2, 3], depth=2)),
        "su_full": ("su", 4, dict(qubits=[0, 1, 2, 3], reps=2, rotations=["rx", "ry"])),
        "su_sub": ("su", 4, dict(qubits=[0, 2, 3], reps=1, rotations=["ry"])),
        "su_rz": ("su", 3, dict(qubits=[0, 1, 2], reps=3, rotations=["rz", "rx"])),
        "budget_cnot": ("budget", 4, dict(param_budget=10, control_gate_spacing=1)),
        "budget_cz": ("budget", 4, dict(param_budget=9, control_gate_spacing=2, control="cz")),
        "budget_sub": ("budget", 5, dict(qubits=[0, 2, 4], param_budget=7, control_gate_spacing=1,
                                         rotations=["ry", "rx", "rz"])),
        "twolocal_6": ("twolocal", 6, dict(qubits=[0, 1, 2, 3, 4, 5], depth=2)),
        "su_6": ("su", 6, dict(qubits=[0, 1, 2, 3, 4, 5], reps=2, rotations=["rx", "ry"])),
        "budget_6": ("budget", 6, dict(param_budget=20, control_gate_spacing=2)),
        **_ansatz_sweep(),
    }


def _ansatz_sweep() -> dict:
    """Random TwoLocal / SU / budget configurations on 2..6 qubits, qubit
    subsets in ascending order."""
    out = {}
    for seed in range(24):
        rng = np.random.default_rng(500 + seed)
        n = int(rng.integers(3, 7))
        kind = ("twolocal", "su", "budget")[seed % 3]
        sub = sorted(int(v) for v in rng.choice(n, int(rng.integers(2, n + 1)), replace=False))
        if kind == "twolocal":
            args = dict(qubits=sub, depth=int(rng.integers(1, 4)))
        elif kind == "su":
            rots = [["rx"], ["ry"], ["rz"], ["rx", "ry"], ["rz", "rx", "ry"]][int(rng.integers(5))]
            args = dict(qubits=sub, reps=int(rng.integers(0, 3)), rotations=rots)
        else:
            args = dict(qubits=sub, param_budget=int(rng.integers(1, 12)),
                        control_gate_spacing=int(rng.integers(1, 4)),
                        rotations=[["rz", "ry"], ["ry"], ["rx", "rz", "ry"]][int(rng.integers(3))])
            if rng.random() < 0.3:
                args["control"] = "cz"
        out[f"sweep_{kind}_{seed}"] = (kind, n, args)
    return out


def build_ansatz(Q, kind: str, n: int, args: dict):
    """A Circuit holding one ansatz of `kind`, built on n qubits."""
    args = dict(args)
    if kind == "twolocal":
        lay = Q.TwoLocal(**args)
    elif kind == "su":
        lay = Q.SU(**args)
    else:
        ctl = Q.CZ if args.pop("control", "cnot") == "cz" else Q.CNOT
        lay = Q.StronglyEntanglingLayerBudget(num_qubits_total=n, control_gate=ctl, remapping=None, **args)
    return Q.Circuit([lay], num_qubits=n)


def ansatz_params(circ) -> list:
    """Deterministic values for the circuit's rotation angles, in parameters() order."""
    k = len(list(circ.parameters()))
    return [round(0.37 * (i + 1) - 1.5 * ((i * 7) % 3), 4) for i in range(k)]


def gate_record(gates) -> list:
    out = []
    for g in gates:
        kind = type(g).__name__.replace("Built", "").lower()
        if kind in ("cnot", "cz"):
            out.append([kind, int(g.c), int(g.t)])
        else:
            out.append([kind, int(g.qubit)])
    return out


def ansatz_cases(qandle):
    """The reference's ansaetze (qandle/ansaetze/): decompositions, parameter
    count and output state for ansatz_params() on a seeded unbatched input
    (the default remapping set to the identity, qw_map.tanh being unpinned)."""
    import qandle.config as ref_config

    out = {}
    saved = ref_config.DEFAULT_MAPPING
    ref_config.DEFAULT_MAPPING = _qw_none
    try:
        for name, (kind, n, args) in ansatz_circuits().items():
            torch.manual_seed(3)
            circ = build_ansatz(qandle, kind, n, args)
            vals = ansatz_params(circ)
            with torch.no_grad():
                for p, v in zip(circ.parameters(), vals):
                    p.fill_(v)
            built = circ.circuit.layers[0]
            rng = np.random.default_rng(11)
            psi = rng.normal(size=(1 << n,)) + 1j * rng.normal(size=(1 << n,))
            psi /= np.linalg.norm(psi)
            with torch.no_grad():
                st = circ(torch.tensor(psi, dtype=torch.cfloat))
            rec = {"params": vals, "built_decompose": gate_record(built.decompose())}
            if kind != "budget":
                rec["unbuilt_decompose"] = gate_record(build_unbuilt_ansatz(qandle, kind, args).decompose())
            out[name] = np.array(json.dumps(rec))
            out[name + "_state"] = st.numpy().astype(np.complex128)
    finally:
        ref_config.DEFAULT_MAPPING = saved
    return out


def build_unbuilt_ansatz(Q, kind: str, args: dict):
    if kind == "twolocal":
        return Q.TwoLocal(**args)
    return Q.SU(**args)


def _qw_none(x):
    return x


MATRIX_QUBITS = 3
MATRIX_NAMED = [0.3, -1.2, 2.0]  # values of the named input "a" for the named rotation
MATRIX_SEED = 5  # torch seed set before each to_matrix call


def matrix_ops(Q) -> dict:
    """name -> built module whose to_matrix() the fixtures pin, for package
    `Q` (the reference or qandle_gb300), on MATRIX_QUBITS qubits.  Call with
    the package's config.DEFAULT_MAPPING set to the identity (qw_map.tanh is
    unpinned).  Rotation angles are fixed after building."""
    n = MATRIX_QUBITS
    m = torch.tensor(workloads.u3_row_matrix(0.3, 1.1, -0.7))
    w = torch.tensor([[[0.1, 0.2, 0.3], [0.4, 0.5, 0.6], [0.7, 0.8, 0.9]],
                      [[-0.2, 1.3, 0.4], [0.9, -1.1, 0.2], [0.5, 0.6, -0.7]]])
    ops = {
        "rx_q0": Q.RX(qubit=0, theta=0.543321, remapping=None),
        "ry_q1": Q.RY(qubit=1, theta=0.543321, remapping=None),
        "rz_q2": Q.RZ(qubit=2, theta=0.543321, remapping=None),
        "rx_named": Q.RX(qubit=1, name="a", remapping=None),
        "u_q1": Q.U(qubit=1, matrix=m),
        "cnot_02": Q.CNOT(0, 2),
        "cnot_20": Q.CNOT(2, 0),
        "cz_12": Q.CZ(1, 2),
        "swap_02": Q.SWAP(a=0, b=2),
        "invert_ry": Q.Invert(Q.RY(qubit=1, theta=0.7, remapping=None).build(num_qubits=n)),
        "invert_u": Q.Invert(Q.U(qubit=2, matrix=m).build(num_qubits=n)),
        "controlled_rx": Q.Controlled(0, Q.RX(qubit=2, theta=0.9, remapping=None)),
        "measure": Q.MeasureProbability(),
        "sel": Q.StronglyEntanglingLayer(qubits=[0, 1, 2], depth=2, q_params=w, remapping=None),
        "sel_sub": Q.StronglyEntanglingLayer(qubits=[0, 2], depth=2, q_params=w[:, :2].clone(), remapping=None),
        "twolocal": Q.TwoLocal(qubits=[0, 1, 2], depth=2),
        "su": Q.SU(qubits=[0, 1, 2], reps=2, rotations=["rx", "ry"]),
    }
    built = {k: v.build(num_qubits=n) for k, v in ops.items()}
    built["budget"] = Q.StronglyEntanglingLayerBudget(num_qubits_total=n, param_budget=7, control_gate_spacing=1,
                                                      rotations=["rz", "ry"], remapping=None)
    built["circuit"] = Q.Circuit([Q.RX(qubit=0, theta=0.4, remapping=None), Q.CNOT(0, 1),
                                  Q.RY(qubit=2, theta=-1.3, remapping=None), Q.U(qubit=1, matrix=m),
                                  Q.CZ(1, 2), Q.SWAP(a=0, b=2), Q.RZ(qubit=1, theta=2.2, remapping=None)],
                                 num_qubits=n)
    for name in ("twolocal", "su", "budget"):
        params = list(built[name].parameters())
        with torch.no_grad():
            for i, p in enumerate(params):
                p.fill_(round(0.37 * (i + 1) - 1.5 * ((i * 7) % 3), 4))
    return built


def state_dict_modules(Q) -> dict:
    """name -> module (package `Q`) whose state_dict layout the fixtures pin.
    Call with Q.config.DEFAULT_MAPPING set to the identity."""
    c1 = Q.Circuit([Q.RX(0, theta=0.1, remapping=None), Q.CNOT(0, 1)], num_qubits=3)
    c2 = Q.Circuit([Q.RY(1, theta=0.2, remapping=None), Q.StronglyEntanglingLayer(qubits=[1, 2], remapping=None)],
                   num_qubits=3)
    return {
        "gates": Q.Circuit([Q.RX(0, theta=0.1, remapping=None), Q.CNOT(0, 1), Q.RY(1, name="a", remapping=None),
                            Q.U(2, matrix=torch.eye(2, dtype=torch.cfloat)), Q.CZ(1, 2), Q.SWAP(a=0, b=2),
                            Q.MeasureProbability()], num_qubits=3),
        "sel": Q.Circuit([Q.AngleEmbedding(name="x", qubits=[0, 1, 2]),
                          Q.StronglyEntanglingLayer(qubits=[0, 1, 2], depth=2, remapping=None),
                          Q.MeasureJointProbability()], num_qubits=3),
        "twolocal": Q.Circuit([Q.TwoLocal(qubits=[0, 1, 2], depth=2)], num_qubits=3),
        "su": Q.Circuit([Q.SU(qubits=[0, 1, 2], reps=2, rotations=["rx", "ry"])], num_qubits=3),
        "budget": Q.Circuit([Q.StronglyEntanglingLayerBudget(num_qubits_total=3, param_budget=5, remapping=None)],
                            num_qubits=3),
        "special": Q.Circuit([Q.Controlled(0, Q.RX(1, theta=0.2, remapping=None)),
                              Q.Invert(Q.RY(2, theta=0.3, remapping=None).build(num_qubits=3)), Q.Reset(1)],
                             num_qubits=3),
        "amplitude": Q.Circuit([Q.AmplitudeEmbedding(name="x", qubits=[0, 1, 2]),
                                Q.RX(0, theta=0.1, remapping=None)], num_qubits=3),
        "split": Q.Circuit([Q.RX(0, theta=0.1, remapping=None), Q.CNOT(0, 1), Q.RY(1, theta=0.2, remapping=None),
                            Q.CNOT(1, 2), Q.RZ(2, theta=0.3, remapping=None)], num_qubits=3).split(max_qubits=2),
        "nested": Q.Circuit([c1, Q.RZ(0, theta=0.4, remapping=None), c2], num_qubits=3),
        "qconv": Q.QConv(in_channels=2, out_channels=3),
    }


def state_dict_cases(qandle):
    """Keys, shapes and dtypes of the reference's state_dicts and
    named_parameters for state_dict_modules(): what a checkpoint saved with
    qandle holds (qcircuit.py, ansaetze/, convolution.py)."""
    import qandle.config as ref_config

    out = {}
    saved = ref_config.DEFAULT_MAPPING
    ref_config.DEFAULT_MAPPING = _qw_none
    try:
        for name, mod in state_dict_modules(qandle).items():
            sd = mod.state_dict()
            rec = {"state_dict": [[k, list(v.shape), str(v.dtype)] for k, v in sd.items()],
                   "parameters": [k for k, _ in mod.named_parameters()]}
            out[name] = np.array(json.dumps(rec))
    finally:
        ref_config.DEFAULT_MAPPING = saved
    return out


def matrix_cases(qandle):
    """to_matrix() of built gates, ansaetze and a circuit (operators.py:60-69,
    ansaetze/ansatz.py:26-33, qcircuit.py:208-212): the inspection half of the
    operator API, including the reference's composition order (utils.reduce_dot
    multiplies later gates from the left) and Controlled returning its
    target's matrix."""
    import qandle.config as ref_config

    out = {}
    saved = ref_config.DEFAULT_MAPPING
    ref_config.DEFAULT_MAPPING = _qw_none
    try:
        for name, mod in matrix_ops(qandle).items():
            kw = {"a": torch.tensor(MATRIX_NAMED)} if name == "rx_named" else {}
            # the budget ansatz builds fresh gates from its unbuilt, angle-less
            # rotations, which draw torch.rand(1) each: seed the draws
            torch.manual_seed(MATRIX_SEED)
            with torch.no_grad():
                mat = mod.to_matrix(**kw)
            out[name] = mat.detach().numpy()
    finally:
        ref_config.DEFAULT_MAPPING = saved
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("QANDLE_REFERENCE_SRC", ""))
    ap.add_argument("--only", default="", help="comma-separated groups to regenerate")
    args = ap.parse_args()
    if not args.reference:
        sys.exit("pass --reference <path to the qandle src directory>")
    qandle = import_reference(args.reference)
    torch.set_num_threads(max(1, os.cpu_count() or 1))
    groups = {
        "gates": gate_cases,
        "embeddings": embedding_cases,
        "measurements": measurement_cases,
        "sel": sel_cases,
        "reupload": reupload_cases,
        "circuits": circuit_cases,
        "random_circuits": random_circuit_cases,
        "random_grads": random_grad_cases,
        "special": special_cases,
        "amplitude": amplitude_cases,
        "amplitude_crop": amplitude_crop_cases,
        "qasm": qasm_cases,
        "splitter": splitter_cases,
        "ansaetze": ansatz_cases,
        "matrices": matrix_cases,
        "state_dicts": state_dict_cases,
    }
    only = [g for g in args.only.split(",") if g]
    for name, fn in groups.items():
        if only and name not in only:
            continue
        arrays = fn(qandle)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **arrays)
        print(f"wrote {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main()

"""Seeded synthetic workloads as plain circuit descriptions.

A description is a dict of plain Python / numpy data, independent of any
executor:

    {"n": int, "batch": int | None,           # None = unbatched state [2^n]
     "gates": [tuple, ...],                   # in application order
     "inputs": {name: np.ndarray},            # named inputs (float32)
     "measure": "probs" | "p0" | "z" | "state" | None,
     "targets": np.ndarray | None}            # MSE targets (adjoint workload)

Gate tuples:

    ("emb", rot, name, qubits)        AngleEmbedding(name, qubits, rotation)
    ("rx"|"ry"|"rz", qubit, theta, name)
                                      theta: float (unnamed) or None (named)
    ("u", qubit, matrix2x2)           qandle.U: the 2x2 is applied as
                                      state @ kron(.., matrix, ..)
    ("cnot", c, t) / ("cz", c, t) / ("swap", a, b)

Seeds follow one convention for every workload: torch.Generator seeded 0 for
inputs, 1 for angles, 2 for targets.  Angles are float32 ~ U(0, 2*pi), inputs
float32 ~ U(0, pi).

The four circuit families are the ones the engine is measured on:

* ``plain_small``   8 qubits, batch 64: AngleEmbedding(rx), 4 x [RY on every
  qubit, CNOT ring i -> i+1 mod 8], joint probabilities.
* ``sel_reupload``  20 qubits, batch 256: AngleEmbedding(rx), 10 strongly
  entangling layers (RZ RY RZ per qubit, CNOT ring of range (layer mod 19)+1,
  the ring of qandle/ansaetze/stronglyentangling.py:106,112-121), named RX
  re-uploading of the inputs on every qubit before layers 0 and 5, <Z> per
  qubit.
* ``adjoint_brick`` 16 qubits, batch 1024: 20 x [RX RY per qubit; CZ on even
  pairs in even layers, CNOT on odd pairs in odd layers], MSE(<Z>, targets).
* ``deep_u``        28 qubits, batch 1: 50 x [U(a,b,c) per qubit; on pairs
  (i, i+1) with i = layer mod 2: CNOT(i -> i+1) then SWAP(i, i+1)], |psi|^2.
"""
from __future__ import annotations

import math

import numpy as np
import torch

TWO_PI = 2.0 * math.pi


def _rand(gen: torch.Generator, *shape, scale: float = 1.0) -> np.ndarray:
    return (torch.rand(*shape, generator=gen, dtype=torch.float32) * scale).numpy()


def _gens():
    return (torch.Generator().manual_seed(0), torch.Generator().manual_seed(1),
            torch.Generator().manual_seed(2))


def u3_row_matrix(a: float, b: float, c: float) -> np.ndarray:
    """Row-vector form of the OpenQASM U(a, b, c).

    qandle applies ``state @ kron(..., matrix, ...)`` (operators.py:101-104,
    :125-126), i.e. the transpose of the matrix acts on column states, so the
    column-form U3 is transposed here.
    """
    ca, sa = math.cos(a / 2.0), math.sin(a / 2.0)
    col = np.array(
        [[ca, -np.exp(1j * c) * sa], [np.exp(1j * b) * sa, np.exp(1j * (b + c)) * ca]],
        dtype=np.complex64,
    )
    return np.ascontiguousarray(col.T)


def plain_small(n: int = 8, batch: int = 64, layers: int = 4) -> dict:
    g_in, g_th, _ = _gens()
    x = _rand(g_in, batch, n, scale=math.pi)
    th = _rand(g_th, layers, n, scale=TWO_PI)
    gates = [("emb", "rx", "x", list(range(n)))]
    for d in range(layers):
        for q in range(n):
            gates.append(("ry", q, float(th[d, q]), None))
        for q in range(n):
            gates.append(("cnot", q, (q + 1) % n))
    return {"name": "plain_small", "n": n, "batch": batch, "gates": gates,
            "inputs": {"x": x}, "measure": "probs", "targets": None}


def sel_reupload(n: int = 20, batch: int = 256, layers: int = 10,
                 reupload_every: int = 5, measure: str = "z") -> dict:
    g_in, g_th, _ = _gens()
    x = _rand(g_in, batch, n, scale=math.pi)
    th = _rand(g_th, layers, n, 3, scale=TWO_PI)
    gates = [("emb", "rx", "x", list(range(n)))]
    inputs = {"x": x}
    for q in range(n):
        inputs[f"up{q}"] = np.ascontiguousarray(x[:, q])
    for d in range(layers):
        if d % reupload_every == 0:
            for q in range(n):
                gates.append(("rx", q, None, f"up{q}"))
        for q in range(n):
            for r, axis in enumerate(("rz", "ry", "rz")):
                gates.append((axis, q, float(th[d, q, r]), None))
        rng = d % (n - 1) + 1
        for q in range(n):
            gates.append(("cnot", q, (q + rng) % n))
    return {"name": "sel_reupload", "n": n, "batch": batch, "gates": gates,
            "inputs": inputs, "measure": measure, "targets": None}


def adjoint_brick(n: int = 16, batch: int = 1024, layers: int = 20) -> dict:
    _, g_th, g_tg = _gens()
    th = _rand(g_th, layers, n, 2, scale=TWO_PI)
    targets = (torch.rand(batch, n, generator=g_tg) * 2.0 - 1.0).numpy().astype(np.float32)
    gates = []
    for d in range(layers):
        for q in range(n):
            gates.append(("rx", q, float(th[d, q, 0]), None))
            gates.append(("ry", q, float(th[d, q, 1]), None))
        if d % 2 == 0:
            for q in range(0, n - 1, 2):
                gates.append(("cz", q, q + 1))
        else:
            for q in range(1, n - 1, 2):
                gates.append(("cnot", q, q + 1))
    return {"name": "adjoint_brick", "n": n, "batch": batch, "gates": gates,
            "inputs": {}, "measure": "z", "targets": targets}


def deep_u(n: int = 28, batch: int = 1, layers: int = 50) -> dict:
    _, g_th, _ = _gens()
    ang = _rand(g_th, layers, n, 3, scale=TWO_PI)
    gates = []
    for d in range(layers):
        for q in range(n):
            a, b, c = (float(v) for v in ang[d, q])
            gates.append(("u", q, u3_row_matrix(a, b, c)))
        for q in range(d % 2, n - 1, 2):
            gates.append(("cnot", q, q + 1))
            gates.append(("swap", q, q + 1))
    return {"name": "deep_u", "n": n, "batch": batch, "gates": gates,
            "inputs": {}, "measure": "probs", "targets": None}


def restrict(desc: dict, n_keep: int) -> dict:
    """Same circuit restricted to qubits 0..n_keep-1 (gates touching a dropped
    qubit are removed).  Used to compare a deep 28-qubit run with a smaller
    prefix circuit."""
    out = []
    for g in desc["gates"]:
        if g[0] == "emb":
            qs = [q for q in g[3] if q < n_keep]
            out.append(("emb", g[1], g[2], qs))
        elif g[0] in ("cnot", "cz", "swap"):
            if g[1] < n_keep and g[2] < n_keep:
                out.append(g)
        elif g[1] < n_keep:
            out.append(g)
    d = dict(desc)
    d["n"] = n_keep
    d["gates"] = out
    return d


def gate_count(desc: dict) -> int:
    """Gates as the reference counts them: an AngleEmbedding over k qubits is
    k rotation gates."""
    c = 0
    for g in desc["gates"]:
        c += len(g[3]) if g[0] == "emb" else 1
    return c


def amp_updates(desc: dict) -> int:
    b = desc["batch"] or 1
    return gate_count(desc) * b * (1 << desc["n"])


def random_sel_request(rng: np.random.Generator, n_range=(4, 24), depth_range=(2, 30),
                       batch_max: int = 512) -> dict:
    """One serving request from the strongly-entangling family: n ~ U{4..24},
    depth ~ U{2..30}, batch log-uniform in [1, 512], angles ~ U(0, 2 pi),
    AngleEmbedding(rx) inputs ~ U(0, pi), <Z> output."""
    n = int(rng.integers(n_range[0], n_range[1] + 1))
    depth = int(rng.integers(depth_range[0], depth_range[1] + 1))
    batch = int(min(batch_max, max(1, round(math.exp(rng.uniform(0.0, math.log(batch_max)))))))
    x = (rng.random((batch, n), dtype=np.float32) * math.pi).astype(np.float32)
    th = (rng.random((depth, n, 3), dtype=np.float32) * TWO_PI).astype(np.float32)
    gates = [("emb", "rx", "x", list(range(n)))]
    for d in range(depth):
        for q in range(n):
            for r, axis in enumerate(("rz", "ry", "rz")):
                gates.append((axis, q, float(th[d, q, r]), None))
        rng_ = d % (n - 1) + 1
        for q in range(n):
            gates.append(("cnot", q, (q + rng_) % n))
    return {"name": "serve_req", "n": n, "batch": batch, "gates": gates,
            "inputs": {"x": x}, "measure": "z", "targets": None}


def build_circuit(desc: dict, engine: str = "fused", **engine_options):
    """qandle_gb300.Circuit for a description, built through the public
    front end exactly as a user would write it."""
    import qandle_gb300 as q

    layers = []
    for g in desc["gates"]:
        k = g[0]
        if k == "emb":
            layers.append(q.AngleEmbedding(name=g[2], qubits=list(g[3]), rotation=g[1]))
        elif k in ("rx", "ry", "rz"):
            cls = {"rx": q.RX, "ry": q.RY, "rz": q.RZ}[k]
            if g[3] is None:
                layers.append(cls(qubit=g[1], theta=torch.tensor(np.float32(g[2])), remapping=None))
            else:
                layers.append(cls(qubit=g[1], name=g[3], remapping=None))
        elif k == "u":
            layers.append(q.U(qubit=g[1], matrix=torch.tensor(np.asarray(g[2], np.complex64))))
        elif k == "cnot":
            layers.append(q.CNOT(control=g[1], target=g[2]))
        elif k == "cz":
            layers.append(q.CZ(control=g[1], target=g[2]))
        elif k == "swap":
            layers.append(q.SWAP(a=g[1], b=g[2]))
        else:
            raise ValueError(f"unknown gate {k}")
    m = desc.get("measure")
    if m == "probs":
        layers.append(q.MeasureJointProbability())
    elif m == "p0":
        layers.append(q.MeasureProbability())
    elif m == "z":
        layers.append(q.MeasureExpectationZ())
    return q.Circuit(layers, num_qubits=desc["n"], engine=engine, **engine_options)


def circuit_inputs(desc: dict, device) -> dict:
    """Named inputs of a description as float32 tensors on `device`."""
    return {k: torch.as_tensor(np.asarray(v, dtype=np.float32)).to(device)
            for k, v in desc.get("inputs", {}).items()}

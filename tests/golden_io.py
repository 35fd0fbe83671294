"""Loading helpers for the golden vectors made by tests/golden/make_golden.py."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"), allow_pickle=False)


def parse_gate(g):
    if g[0] == "u":
        m = np.array([complex(a, b) for a, b in g[2]], dtype=np.complex64).reshape(2, 2)
        return ("u", g[1], m)
    if g[0] == "emb":
        return ("emb", g[1], g[2], list(g[3]))
    if g[0] in ("rx", "ry", "rz"):
        return (g[0], g[1], None if g[2] is None else float(g[2]), g[3])
    return tuple(g)


def circuit_desc(z, name):
    d = json.loads(str(z[f"{name}_desc"]))
    d["gates"] = [parse_gate(g) for g in d["gates"]]
    d["inputs"] = {k: z[f"{name}_in_{k}"] for k in d.pop("input_names")}
    d["targets"] = z[f"{name}_targets"] if f"{name}_targets" in z.files else None
    return d


# ---- Invert / Controlled / Reset cases (special.npz) ----


def _u(spec_m):
    return np.array([complex(a, b) for a, b in spec_m], dtype=np.complex64).reshape(2, 2)


def special_gates(spec, inputs=None):
    """Oracle description gates of one special.npz spec (Invert as the
    inverse gate, Controlled as controlled kinds, Reset as reset)."""
    op = spec["op"]
    if op == "reset":
        return [("reset", spec["qubit"])]
    if op == "invert":
        t = spec["target"]
        if t[0] in ("rx", "ry", "rz"):
            return [(t[0], t[1], -float(t[2]), None)]
        if t[0] == "u":
            return [("u", t[1], np.linalg.inv(_u(t[2]).astype(np.complex128)).astype(np.complex64))]
        return [tuple(t)]
    if op == "controlled":
        t = spec["target"]
        if t[0] == "u":
            return [("cu", spec["control"], t[1], _u(t[2]))]
        name = t[3] if len(t) > 3 else None
        return [("c" + t[0], spec["control"], t[1], None if t[2] is None else float(t[2]), name)]
    if op == "circuit":
        out = []
        for lay in spec["layers"]:
            if lay[0] == "controlled":
                out += special_gates({"op": "controlled", "control": lay[1], "target": lay[2]})
            elif lay[0] == "invert":
                out += special_gates({"op": "invert", "target": lay[1]})
            elif lay[0] in ("rx", "ry", "rz"):
                out.append((lay[0], lay[1], float(lay[2]), None))
            else:
                out.append(tuple(lay))
        return out
    raise ValueError(op)


def special_layers(q, spec, n):
    """The same spec built with the qandle_gb300 front end (``q`` = the package)."""
    rot = {"rx": q.RX, "ry": q.RY, "rz": q.RZ}

    def target(t):
        if t[0] in rot:
            if len(t) > 3 and t[3] is not None:
                return rot[t[0]](qubit=t[1], name=t[3], remapping=None)
            return rot[t[0]](qubit=t[1], theta=float(t[2]), remapping=None)
        if t[0] == "u":
            import torch
            return q.U(qubit=t[1], matrix=torch.tensor(_u(t[2])))
        cls = {"cnot": q.CNOT, "cz": q.CZ, "swap": q.SWAP}[t[0]]
        return cls(t[1], t[2]) if t[0] != "swap" else cls(a=t[1], b=t[2])

    op = spec["op"]
    if op == "reset":
        return [q.Reset(qubit=spec["qubit"])]
    if op == "invert":
        return [q.Invert(target(spec["target"]).build(num_qubits=n))]
    if op == "controlled":
        return [q.Controlled(spec["control"], target(spec["target"]))]
    if op == "circuit":
        out = []
        for lay in spec["layers"]:
            if lay[0] == "controlled":
                out.append(q.Controlled(lay[1], target(lay[2])))
            elif lay[0] == "invert":
                out.append(q.Invert(target(lay[1]).build(num_qubits=n)))
            else:
                out.append(target(lay))
        return out
    raise ValueError(op)

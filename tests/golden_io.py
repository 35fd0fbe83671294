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

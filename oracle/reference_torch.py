"""The reference's own torch path (gstenzel/qandle 0.1.8) as a CPU baseline
and as the other side of the drop-in boundary tests.

Test and benchmark infrastructure: imported by bench.py's CPU baselines and
by tests, never by the qandle_gb300 package.  The reference is imported from
the copy that oracle/install_reference.sh puts into baseline/_ref (or from a
source tree given as `path`).  Two of its dependencies are not in the offline
images and get stand-ins at import time:

* qw_map (qw-map 0.1.2): `none` is the identity, which is what
  `remapping=None` means; `tanh` raises (it is never used here);
* networkx, when absent: only the reference's circuit splitter uses it, so
  the stand-in lets the package import and raises if a graph is built.

The circuits are built from the reference's own layer classes, exactly as a
user of the reference writes them (qandle/qcircuit.py:13-60), and run
through its Circuit.forward (qcircuit.py:163-174) on the host CPU.
"""
from __future__ import annotations

import importlib.util
import os
import sys
import types

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DIR = os.path.join(ROOT, "baseline", "_ref")


def _stand_ins() -> None:
    if "qw_map" not in sys.modules and importlib.util.find_spec("qw_map") is None:
        qw = types.ModuleType("qw_map")
        qw.none = lambda x: x

        def tanh(x):
            raise RuntimeError("qw_map.tanh stand-in: only remapping=None is used with the reference here")

        qw.tanh = tanh
        sys.modules["qw_map"] = qw
    if "networkx" not in sys.modules and importlib.util.find_spec("networkx") is None:
        nx = types.ModuleType("networkx")

        class _Unavailable:
            def __init__(self, *a, **k):
                raise RuntimeError("networkx is not installed: the reference's splitter cannot run here")

        nx.__getattr__ = lambda name: _Unavailable  # annotations such as nx.DiGraph resolve
        sys.modules["networkx"] = nx


def unavailable_reason(path: str | None = None) -> str | None:
    """None when the reference can be imported from `path` (default
    baseline/_ref), else a one-line reason."""
    p = path or REF_DIR
    if not os.path.isdir(os.path.join(p, "qandle")):
        return f"the reference is not installed in {os.path.relpath(p, ROOT)} (run oracle/install_reference.sh)"
    try:
        import_reference(p)
    except Exception as e:  # noqa: BLE001 - report any import failure as the reason
        return f"importing the reference failed: {type(e).__name__}: {e}"
    return None


def import_reference(path: str | None = None):
    """The reference package `qandle` (imported once per process)."""
    if "qandle" in sys.modules:
        return sys.modules["qandle"]
    p = path or REF_DIR
    _stand_ins()
    if p not in sys.path:
        sys.path.insert(0, p)
    import qandle  # noqa: F401

    return sys.modules["qandle"]


def build_circuit(qandle, desc: dict):
    """A reference Circuit for a circuit description (see
    qandle_gb300.workloads): its layers are the reference's classes with the
    description's angles, inputs are named, remapping=None."""
    import torch

    layers = []
    for g in desc["gates"]:
        k = g[0]
        if k == "emb":
            layers.append(qandle.AngleEmbedding(name=g[2], qubits=list(g[3]), rotation=g[1]))
        elif k in ("rx", "ry", "rz"):
            cls = {"rx": qandle.RX, "ry": qandle.RY, "rz": qandle.RZ}[k]
            if g[3] is None:
                layers.append(cls(qubit=g[1], theta=torch.tensor(np.float32(g[2])), remapping=None))
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
        else:
            raise ValueError(f"unknown gate {k}")
    m = desc.get("measure")
    if m == "probs":
        layers.append(qandle.MeasureJointProbability())
    elif m in ("p0", "z"):
        layers.append(qandle.MeasureProbability())
    return qandle.Circuit(layers, num_qubits=desc["n"])


def inputs(desc: dict) -> dict:
    import torch

    return {k: torch.tensor(np.asarray(v, dtype=np.float32)) for k, v in desc.get("inputs", {}).items()}

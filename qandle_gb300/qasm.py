"""OpenQASM export (mirrors qandle/qasm.py:1-70) and ingest.

Export keeps the reference's text format, since that is what its users get
from ``Circuit.to_openqasm2()`` / ``to_openqasm3()``: one
QasmRepresentation per gate, rendered as ``gate(value) q[i];``, and the
same headers.  Ingest (``parse``) reads the gate subset this engine runs from
OpenQASM 2 or 3 text -- rx/ry/rz with a value or a named input, cx, cz,
swap, reset, U-gate definitions as exported, measure lines -- into
qandle_gb300 layers, so circuits can arrive as text (e.g. serving
requests).
"""
from __future__ import annotations

import dataclasses
import math
import re
import typing

__all__ = ["QasmRepresentation", "convert_to_qasm", "parse"]


@dataclasses.dataclass
class QasmRepresentation:
    """One gate of a circuit in OpenQASM (qasm.py:5-31)."""

    gate_str: str
    gate_value: typing.Union[str, float] = ""
    qubit: typing.Union[str, int] = ""
    qasm3_inputs: str = ""
    qasm3_outputs: str = ""

    def __iter__(self):
        yield self

    def to_string(self) -> str:
        s = self.gate_str
        if self.qasm3_inputs != "":
            s += f"({self.qasm3_inputs})"
        elif self.gate_value != "":
            s += f"({self.gate_value})"
        if self.qubit != "" and self.qubit is not None:
            s += f" q[{self.qubit}]"
        return s + ";"


def convert_to_qasm(circuit, qasm_version: int = 2, include_header: bool = True) -> str:
    """OpenQASM text of a circuit (qasm.py:34-70)."""
    num_qubits = circuit.num_qubits
    if qasm_version == 2:
        header = f"OPENQASM 2.0;\ninclude \"qelib1.inc\";\nqreg q[{num_qubits}];\ncreg c[{num_qubits}];\n"
    else:
        header = f"OPENQASM 3.0;\nqubit[{num_qubits}] q;\nbit[{num_qubits}] c;\n"
    reps = circuit.to_qasm()
    out = header if include_header else ""
    if qasm_version == 3:
        for rep in reps:
            for r in rep:
                if r.qasm3_inputs != "":
                    out += f"input float {r.qasm3_inputs};\n"
                if r.qasm3_outputs != "":
                    out += f"output float {r.qasm3_outputs};\n"
    for rep in reps:
        for r in rep:
            out += r.to_string() + "\n"
    return out


_NUM = r"[-+0-9.eE]+(?:\s*\*\s*pi|pi\s*/\s*[0-9.]+)?"


def _value(txt: str) -> float:
    t = txt.replace(" ", "").replace("pi", str(math.pi))
    if not re.fullmatch(r"[-+0-9.eE*/]+", t):
        raise ValueError(f"unsupported angle expression {txt!r}")
    return float(eval(t, {"__builtins__": {}}, {}))  # digits, dots, signs, * and / only


def parse(text: str):
    """Layers (qandle_gb300 operators and a final measurement) and the qubit
    count of an OpenQASM 2/3 program in the supported subset.  Named angles
    (``rx(x0) q[0];`` with ``input float x0;``) become named rotations."""
    from . import measurements, operators

    n = None
    inputs = set()
    layers = []
    measured = set()
    defs = {}  # exported U gate definitions: name -> 2x2
    for raw in text.splitlines():
        line = raw.split("//")[0].strip()
        if not line or line.startswith(("OPENQASM", "include", "creg", "bit[")):
            continue
        m = re.fullmatch(r"qreg\s+q\[(\d+)\];", line) or re.fullmatch(r"qubit\[(\d+)\]\s+q;", line)
        if m:
            n = int(m.group(1))
            continue
        m = re.fullmatch(r"input\s+float\s+(\w+);", line)
        if m:
            inputs.add(m.group(1))
            continue
        if line.startswith("output "):
            continue
        m = re.fullmatch(r"gate\s+(\w+)\s+q\[(\d+)\]\s*\{\{?\s*U\(([^)]*)\)\s*\}?\}\s*q\[(\d+)\];", line)
        if m:
            import torch

            vals = [complex(v.strip().replace("j", "j")) for v in m.group(3).split(",")]
            mat = torch.tensor(vals, dtype=torch.complex64).reshape(2, 2)
            layers.append(operators.U(qubit=int(m.group(4)), matrix=mat))
            continue
        m = re.fullmatch(r"(rx|ry|rz)\(([^)]*)\)\s*q\[(\d+)\];", line)
        if m:
            cls = {"rx": operators.RX, "ry": operators.RY, "rz": operators.RZ}[m.group(1)]
            arg, q = m.group(2).strip(), int(m.group(3))
            if arg in inputs or re.fullmatch(r"[A-Za-z_]\w*", arg):
                layers.append(cls(qubit=q, name=arg, remapping=None))
            else:
                layers.append(cls(qubit=q, theta=_value(arg), remapping=None))
            continue
        m = re.fullmatch(r"(cx|cz|swap)\s+q\[(\d+)\],\s*q\[(\d+)\];", line)
        if m:
            a, b = int(m.group(2)), int(m.group(3))
            if m.group(1) == "cx":
                layers.append(operators.CNOT(a, b))
            elif m.group(1) == "cz":
                layers.append(operators.CZ(a, b))
            else:
                layers.append(operators.SWAP(a=a, b=b))
            continue
        m = re.fullmatch(r"reset\s+q\[(\d+)\];", line)
        if m:
            layers.append(operators.Reset(qubit=int(m.group(1))))
            continue
        m = re.fullmatch(r"measure\s+q\[(\d+)\]\s*->\s*c\[(\d+)\];", line) or \
            re.fullmatch(r"c\[(\d+)\]\s*=\s*measure\s+q\[(\d+)\];", line)
        if m:
            measured.add(int(m.group(1)))
            continue
        raise ValueError(f"unsupported OpenQASM line: {raw!r}")
    if n is None:
        raise ValueError("no qubit register declared")
    if measured:
        layers.append(measurements.MeasureProbability())
    return layers, n

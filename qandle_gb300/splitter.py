"""Circuit splitter (mirrors qandle/splitter/main.py and splitter/grouping.py).

``split(circuit, max_qubits)`` cuts a circuit into subcircuits of at most
``max_qubits`` qubits the way the reference does, and returns the same
structure: ``{group: SubcircuitContainer(layers, mapping)}``, where
``mapping`` sends each original qubit of the group to its index inside the
subcircuit and ``layers`` are new gates on those indices.

The algorithm is the reference's, restated without networkx:

1. Every CNOT of the decomposed circuit is a node; a CNOT depends on the
   previous CNOT it shares a qubit with (main.py:27-55).
2. Groups grow greedily (grouping.py:24-64): the first ungrouped node with the
   fewest distinct predecessors starts a group, and a depth-first walk over
   successors adds every ungrouped node whose predecessors are all grouped
   while the group stays within ``max_qubits`` qubits.
3. Every other gate joins the group of the nearest earlier CNOT on its qubit,
   or of the next one when there is none (main.py:58-104).
4. Each group's qubits are renumbered in ascending order (main.py:113-157).

The fused engine does not need the cut to bound memory (its planner already
works tile by tile); a split circuit runs its subcircuits' gates, mapped
back to the original qubits, as one fused program (qandle_gb300.qcircuit).
"""
from __future__ import annotations

import dataclasses
import typing

from . import operators as op

__all__ = ["split", "SubcircuitContainer"]

_CNOT_TYPES = (op.CNOT, op.BuiltCNOT)


@dataclasses.dataclass
class SubcircuitContainer:
    layers: list  # gates on the subcircuit's qubit indices
    mapping: dict  # original qubit -> subcircuit qubit


class _Node:
    """One CNOT of the circuit (grouping.py:5-18)."""

    __slots__ = ("c", "t", "index", "group", "succ", "pred")

    def __init__(self, c: int, t: int, index: int):
        self.c = c
        self.t = t
        self.index = index
        self.group = -1
        self.succ: typing.List["_Node"] = []  # in order of first edge insertion
        self.pred: typing.List["_Node"] = []

    def __repr__(self) -> str:
        return f"{self.c}|{self.t}"


def split(circuit, max_qubits: int = 5) -> typing.Dict[int, SubcircuitContainer]:
    """Subcircuits of at most `max_qubits` qubits (main.py:12-24)."""
    assert circuit.num_qubits > 1, "Can't split circuits with only 1 qubit"
    assert all(isinstance(layer, op.Operator) for layer in circuit.layers), (
        f"Unknown layer type in circuit: "
        f"{[type(layer) for layer in circuit.layers if not isinstance(layer, op.Operator)]}")
    nodes = _construct_graph(circuit)
    _group_nodes(nodes, max_qubits)
    assigned = _assign_to_subcircuits(nodes, list(circuit.layers))
    return {i: _normalize_subcircuit(layers) for i, layers in assigned.items()}


def _construct_graph(circuit) -> typing.List[_Node]:
    """CNOT nodes with edges to the next CNOT on each qubit (main.py:27-55)."""
    decomposed = circuit.decompose()
    nodes = [_Node(layer.c, layer.t, i) for i, layer in enumerate(decomposed.layers)
             if isinstance(layer, _CNOT_TYPES)]
    assert len(nodes) > 0, (
        "No CNOTs in the circuit, instead of splitting, just use separate circuits for each qubit")
    used = set(n.c for n in nodes) | set(n.t for n in nodes)
    assert len(used) == circuit.num_qubits, (
        "Circuit has qubits not used in CNOTs. Instead of splitting, just use separate circuits "
        f"for separate qubits. Only used qubits are: {used}")
    per_qubit: typing.Dict[int, typing.List[_Node]] = {w: [] for w in range(circuit.num_qubits)}
    for n in nodes:
        per_qubit[n.c].append(n)
        per_qubit[n.t].append(n)
    for w in range(circuit.num_qubits):
        chain = per_qubit[w]
        for a, b in zip(chain, chain[1:]):
            if b not in a.succ:  # a directed graph keeps one edge per pair
                a.succ.append(b)
                b.pred.append(a)
    return nodes


def _group_nodes(nodes: typing.List[_Node], max_qubits: int) -> None:
    """Greedy grouping (grouping.py:31-64); the walk over successors is the
    reference's recursive depth-first order, kept on an explicit stack."""
    assert max_qubits >= 2, "max_qubits must be >= 2"
    by_in_degree = sorted(nodes, key=lambda n: len(n.pred))  # stable: circuit order on ties
    next_group = 0
    while True:
        first = next((n for n in by_in_degree if n.group == -1), None)
        if first is None:
            return
        first.group = next_group
        next_group += 1
        used = {first.c, first.t}
        stack = [(first, iter(first.succ))]
        while stack:
            start, succ = stack[-1]
            n = next(succ, None)
            if n is None:
                stack.pop()
                continue
            if (n.group == -1 and all(p.group != -1 for p in n.pred)
                    and len(used | {n.c, n.t}) <= max_qubits):
                n.group = start.group
                used.add(n.c)
                used.add(n.t)
                stack.append((n, iter(n.succ)))


def _assign_to_subcircuits(nodes: typing.List[_Node], layers: list) -> typing.Dict[int, list]:
    """Gates of each group in circuit order (main.py:58-104)."""
    groups: typing.Dict[int, typing.Dict[int, object]] = {g: {} for g in sorted(set(n.group for n in nodes))}
    node_at = {n.index: n for n in nodes}
    cnot_at = [i for i, layer in enumerate(layers) if isinstance(layer, _CNOT_TYPES)]
    for i in cnot_at:
        groups[node_at[i].group][i] = layers[i]
    for i, layer in enumerate(layers):
        if isinstance(layer, _CNOT_TYPES):
            continue
        w = layer.qubit
        prev = nxt = None
        for j in cnot_at:
            if layers[j].c == w or layers[j].t == w:
                if j < i:
                    prev = j
                elif j > i:
                    nxt = j
                    break
        near = prev if prev is not None else nxt
        assert near is not None, f"no CNOT touches qubit {w} of layer {i} ({layer})"
        groups[node_at[near].group][i] = layer
    return {g: [gates[i] for i in sorted(gates)] for g, gates in groups.items()}


def _normalize_subcircuit(gates: list) -> SubcircuitContainer:
    """Renumber a group's qubits to 0..m-1 in ascending order (main.py:113-157).
    The new gates are fresh unbuilt gates carrying theta and name only, as in
    the reference (a rotation's remapping is the default one)."""
    qubits = set()
    for g in gates:
        if isinstance(g, _CNOT_TYPES):
            qubits.update((g.c, g.t))
        else:
            qubits.add(g.qubit)
    mapping = {q: i for i, q in enumerate(sorted(qubits))}
    new_layers = []
    for g in gates:
        if isinstance(g, _CNOT_TYPES):
            new_layers.append(op.CNOT(control=mapping[g.c], target=mapping[g.t]))
        elif isinstance(g, op.BuiltU):
            new_layers.append(op.BuiltU(qubit=mapping[g.qubit], matrix=g.original_matrix,
                                        num_qubits=len(qubits), self_description=g.description))
        else:
            cls = op.BUILT_CLASS_RELATION.T[type(g)] if isinstance(g, op.BuiltOperator) else type(g)
            other = {}
            if getattr(g, "theta", None) is not None:
                other["theta"] = g.theta
            if getattr(g, "name", None) is not None:
                other["name"] = g.name
            new_layers.append(cls(qubit=mapping[g.qubit], **other))
    return SubcircuitContainer(new_layers, mapping)

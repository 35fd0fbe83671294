"""StronglyEntanglingLayer (mirrors qandle/ansaetze/stronglyentangling.py).

Rotations ``rotations`` on every listed qubit per layer, then a CNOT ring of
range (layer mod (len(qubits)-1)) + 1 (stronglyentangling.py:96-121).  It
decomposes into the gate layers of qandle_gb300.operators, so both engines
run it without a kernel of its own.
"""
from __future__ import annotations

import copy
import typing

import torch

from . import config, remap
from . import operators as op
from .embeddings import parse_rot

__all__ = ["StronglyEntanglingLayer", "StronglyEntanglingLayerBuilt"]

_ROT_CLASS = {0: op.RX, 1: op.RY, 2: op.RZ}


class StronglyEntanglingLayer(op.UnbuiltOperator):
    def __init__(self, qubits: typing.List[int], num_qubits_total: typing.Union[int, None] = None,
                 depth: int = 1, rotations=("rz", "ry", "rz"), q_params=None,
                 remapping: typing.Union[typing.Callable, None] = config.DEFAULT_MAPPING):
        self.depth = depth
        self.qubits = qubits
        self.num_qubits = num_qubits_total
        self.rots = [_ROT_CLASS[parse_rot(r)] for r in rotations]
        if q_params is None:
            q_params = torch.rand(depth, len(qubits), len(rotations))
        self.q_params = q_params
        self.remapping = remap.none if remapping is None else remapping

    def build(self, *args, **kwargs) -> "StronglyEntanglingLayerBuilt":
        return StronglyEntanglingLayerBuilt(num_qubits=kwargs["num_qubits"], depth=self.depth,
                                            rotations=self.rots, q_params=self.q_params,
                                            remapping=self.remapping, qubits=self.qubits)

    def __str__(self) -> str:
        return "SEL"

    def decompose(self) -> typing.List[op.UnbuiltOperator]:
        layers = []
        for d in range(self.depth):
            for wi, w in enumerate(self.qubits):
                for r in range(len(self.rots)):
                    layers.append(self.rots[r](qubit=w, theta=self.q_params[d, wi, r],
                                               remapping=self.remapping))
            layers.extend(StronglyEntanglingLayerBuilt._get_cnots(
                self.qubits, self.num_qubits, d % (len(self.qubits) - 1), build=False))
        return layers


class StronglyEntanglingLayerBuilt(op.BuiltOperator):
    def __init__(self, num_qubits: int, qubits: typing.List[int], depth: int, rotations,
                 q_params: torch.Tensor, remapping):
        super().__init__()
        self.num_qubits = num_qubits
        self.depth = depth
        self.rots = rotations
        self.qubits = qubits
        layers = []
        for d in range(depth):
            for wi, w in enumerate(self.qubits):
                for r in range(len(self.rots)):
                    layers.append(self.rots[r](qubit=w, theta=q_params[d, wi, r],
                                               remapping=remapping).build(num_qubits))
            layers.extend(self._get_cnots(self.qubits, self.num_qubits, d % (len(self.qubits) - 1)))
        self.mods = torch.nn.Sequential(*layers)

    def forward(self, state: torch.Tensor):
        return self.mods(state)

    @staticmethod
    def _get_cnots(qubits, num_qubits_total, iteration, build=True):
        assert iteration + 1 < num_qubits_total
        cnots = []
        for ci in range(len(qubits)):
            ti = (ci + iteration + 1) % len(qubits)
            g = op.CNOT(qubits[ci], qubits[ti])
            cnots.append(g.build(num_qubits_total) if build else g)
        return cnots

    def __str__(self) -> str:
        return "SEL"

    def decompose(self):
        return [copy.deepcopy(m) for m in self.mods]

    def to_qasm(self):
        return [g.to_qasm() for g in self.decompose()]

    def to_matrix(self, **kwargs):
        m = None
        for mod in self.mods:
            mm = mod.to_matrix(**kwargs)
            m = mm if m is None else m @ mm
        return m

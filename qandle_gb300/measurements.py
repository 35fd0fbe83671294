"""Measurements (mirrors qandle/measurements.py:12-126).

MeasureProbability gives P(qubit q = 0) per sample with the reference's
output shapes, including its squeeze (measurements.py:120-123): a batch of
one gives [n], one qubit gives [B].  MeasureAllAbsolute (alias
MeasureJointProbability) gives |psi|^2.  MeasureExpectationZ has no
counterpart in the reference: <Z_q> = P0_q - P1_q, which equals
2 * MeasureProbability - 1 for a normalised state.
"""
from __future__ import annotations

import random

import torch

from . import operators as op
from . import plain

__all__ = ["BuiltMeasurement", "UnbuiltMeasurement", "MeasureAllAbsolute", "MeasureJointProbability",
           "MeasureState", "MeasureProbability", "MeasureProbabilityBuilt", "MeasureExpectationZ",
           "MeasureExpectationZBuilt"]


class BuiltMeasurement(op.BuiltOperator):
    def __str__(self) -> str:
        return "M"

    def to_qasm(self):
        """measure q[w] -> c[w] for every qubit (measurements.py:16-22)."""
        from . import qasm

        i = hash(random.random())
        return [qasm.QasmRepresentation(gate_str=f"measure q[{w}] -> c[{w}]", qasm3_outputs=f"measured_{i}_{w}")
                for w in range(self.num_qubits)]

    def to_matrix(self):
        return torch.eye(2 ** self.num_qubits)


class UnbuiltMeasurement(op.UnbuiltOperator):
    def __str__(self) -> str:
        return "M"

    def build(self, num_qubits: int, **kwargs) -> BuiltMeasurement:
        return BUILT_CLASS_RELATION[self.__class__](num_qubits=num_qubits, **kwargs)


class MeasureAllAbsolute(BuiltMeasurement):
    """|psi|^2 (measurements.py:73-79)."""

    def forward(self, state: torch.Tensor) -> torch.Tensor:
        return plain.Probs.apply(state)


MeasureJointProbability = MeasureAllAbsolute


class MeasureState(BuiltMeasurement):
    """Identity (measurements.py:85-91)."""

    def forward(self, state: torch.Tensor) -> torch.Tensor:
        return state


class MeasureProbability(UnbuiltMeasurement):
    r"""Probability of each qubit being in |0> (measurements.py:94-98)."""


def _reference_shape(p0_bn: torch.Tensor) -> torch.Tensor:
    """[B, n] -> the reference's output: sum over [n, B] then squeeze() and
    transpose(-1, 0) (measurements.py:123)."""
    return p0_bn.transpose(0, 1).squeeze().transpose(-1, 0)


class MeasureProbabilityBuilt(BuiltMeasurement):
    def __init__(self, num_qubits: int):
        super().__init__()
        self.num_qubits = num_qubits
        self.qubits = list(range(num_qubits))

    def forward(self, state: torch.Tensor):
        p0 = plain.MeasureP0.apply(state, self.num_qubits)
        return _reference_shape(p0)


class MeasureExpectationZ(UnbuiltMeasurement):
    r"""<Z_q> per qubit: P(q = 0) - P(q = 1).  Not in the reference."""


class MeasureExpectationZBuilt(BuiltMeasurement):
    def __init__(self, num_qubits: int):
        super().__init__()
        self.num_qubits = num_qubits

    def forward(self, state: torch.Tensor):
        p0 = plain.MeasureP0.apply(state, self.num_qubits)
        norm = plain.Probs.apply(state).reshape(-1, 2 ** self.num_qubits).sum(-1, keepdim=True)
        return _reference_shape(2.0 * p0 - norm)


BUILT_CLASS_RELATION = {MeasureProbability: MeasureProbabilityBuilt,
                        MeasureExpectationZ: MeasureExpectationZBuilt}

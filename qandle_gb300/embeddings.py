"""AngleEmbedding (mirrors qandle/embeddings.py:114-214).

The reference forms the per-sample product of n dense 2^n x 2^n rotation
matrices and applies it to |0..0>.  The product of rotations on distinct
qubits is the product state prod_q R_q(x_q)|0>, which the CUDA kernel writes
directly (8 bytes per amplitude, no matmuls).
"""
from __future__ import annotations

import random
import typing

import torch

from . import operators as op
from . import plain

__all__ = ["AngleEmbedding", "AngleEmbeddingBuilt", "AmplitudeEmbedding", "AmplitudeEmbeddingBuilt",
           "InputOperator", "InputOperatorBuilt"]

_ROT = {"x": 0, "y": 1, "z": 2}


def parse_rot(rot: str) -> int:
    """Axis index of 'rx'/'x'/'ry'/... (utils.parse_rot, qandle/utils.py:26-37)."""
    r = rot.lower().replace("r", "")
    if r not in _ROT:
        raise ValueError(f"Unknown rotation {rot}")
    return _ROT[r]


class InputOperator(op.UnbuiltOperator):
    ...


class InputOperatorBuilt(op.BuiltOperator):
    def decompose(self):
        raise NotImplementedError(f"Decomposing {self.__class__} is not yet supported")

    def to_matrix(self):
        raise ValueError("Input operators do not have a matrix representation")


class AngleEmbeddingBuilt(InputOperatorBuilt):
    """Ignores the incoming state and writes the embedded product state."""

    def __init__(self, name: str, num_qubits: int, qubits: typing.List[int], rotation: str):
        super().__init__()
        self.num_qubits = num_qubits
        self.qubits = list(qubits)
        self.named = True
        self.name = name
        self.rotation = rotation
        self.axis = parse_rot(rotation)
        for q in self.qubits:
            if not 0 <= q < num_qubits:
                raise ValueError(f"embedded qubit {q} out of range for {num_qubits} qubits")

    def forward(self, state=None, **kwargs):
        inp = torch.as_tensor(kwargs[self.name])
        out = plain.AngleEmbed.apply(inp, self.num_qubits, self.qubits, self.axis)
        if inp.dim() == 1:
            return out.reshape(1 << self.num_qubits)
        return out.reshape(*inp.shape[:-1], 1 << self.num_qubits)

    def __str__(self) -> str:
        return f"AngleEmbedding_{self.rotation}"

    def to_qasm(self):
        """One named rotation per embedded qubit (embeddings.py:166-171)."""
        rot = {0: op.RX, 1: op.RY, 2: op.RZ}[self.axis]
        r = hash(random.random())
        return [rot(qubit=w, name=f"angle_{r}_{w}").to_qasm() for w in self.qubits]


class AngleEmbedding(InputOperator):
    """Angle embedding of named inputs (embeddings.py:184-214)."""

    def __init__(self, name: str, qubits: typing.Union[typing.List[int], None] = None,
                 rotation="rx"):
        self.name = name
        self.named = True
        self.qubits = qubits
        self.rotation = rotation

    def build(self, num_qubits: int, **kwargs) -> AngleEmbeddingBuilt:
        qubits = list(range(num_qubits)) if self.qubits is None else self.qubits
        return AngleEmbeddingBuilt(name=self.name, qubits=qubits, num_qubits=num_qubits,
                                   rotation=self.rotation)

    def __str__(self) -> str:
        return f"AngleEmbedding_{self.rotation}"


class AmplitudeEmbeddingBuilt(InputOperatorBuilt):
    """Ignores the incoming state and sets the features as the state
    (embeddings.py:29-66): padded with ``pad_with`` to 2^n entries,
    optionally normalised, imaginary part 0."""

    def __init__(self, name: str, num_qubits: int, normalize: bool, pad_with: typing.Union[float, None]):
        super().__init__()
        self.num_qubits = num_qubits
        self.normalize = bool(normalize)
        self.pad_with = pad_with
        self.named = True
        self.name = name

    def forward(self, _=None, **kwargs):
        x = torch.as_tensor(kwargs[self.name])
        return plain.AmpEmbed.apply(x, self.num_qubits, self.pad_with, self.normalize)

    def __str__(self) -> str:
        return "AmplitudeEmbedding"


class AmplitudeEmbedding(InputOperator):
    """Amplitude embedding of a named input (embeddings.py:69-111)."""

    def __init__(self, name: str, qubits: list, normalize: bool = False,
                 pad_with: typing.Union[float, None] = None):
        self.name = name
        self.named = True
        self.qubits = qubits
        self.pad_with = pad_with
        self.normalize = normalize

    def build(self, num_qubits: int, **kwargs) -> AmplitudeEmbeddingBuilt:
        assert num_qubits == len(self.qubits), "Current Implementation requires all qubits to be used."
        return AmplitudeEmbeddingBuilt(num_qubits=num_qubits, normalize=self.normalize, pad_with=self.pad_with,
                                       name=self.name)

    def __str__(self) -> str:
        return "AmplitudeEmbedding"

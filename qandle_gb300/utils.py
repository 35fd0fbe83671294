"""Small helpers of qandle's public API (mirrors qandle/utils.py:1-70).

* ``reduce_dot(*mats)``: the product of a chain of (batched) matrices, later
  matrices applied last (utils.py:6-22).
* ``parse_rot(name)``: "rx" / "RY" / "z" ... -> the rotation class (utils.py:25-37).
* ``do_not_implement(*names, reason="")``: a metaclass that refuses class
  bodies defining any of `names` (utils.py:40-51).
* ``get_matrix_transforms(n, qubits)``: a pair of modules moving a state
  ``[B, 2^n]`` to the view ``[(B * 2^(n-m)), 2^m]`` in which `qubits` (in the
  given order) form the fast axis, and back (utils.py:54-70).  The reference
  builds them with einops; these are plain reshape/permute modules with the
  same index mapping.
"""
from __future__ import annotations

import typing

import torch

__all__ = ["reduce_dot", "parse_rot", "do_not_implement", "get_matrix_transforms"]


def reduce_dot(*args):
    """M_k @ ... @ M_1 @ M_0 for args (M_0, ..., M_k); 2-D factors act as a
    batch of one, a single argument is returned as it is."""
    if len(args) == 1:
        return args[0]
    out = args[0].unsqueeze(0) if args[0].dim() == 2 else args[0]
    for m in args[1:]:
        if m.dim() == 2:
            m = m.unsqueeze(0)
        elif m.dim() != 3:
            raise ValueError(f"Invalid shape {m.shape}")
        out = torch.matmul(m, out)
    return out


def parse_rot(rot: str):
    """Rotation class for a name such as "rx", "RY" or "z"."""
    from . import operators

    key = rot.lower().replace("r", "")
    classes = {"x": operators.RX, "y": operators.RY, "z": operators.RZ}
    if key not in classes:
        raise ValueError(f"Unknown rotation {key}")
    return classes[key]


def do_not_implement(*protected, reason: str = "") -> type:
    """Metaclass refusing class bodies that define any `protected` name."""

    class LimitedClass(type):
        def __new__(mcs, name, bases, attrs):
            for attribute in attrs:
                if attribute in protected:
                    raise AttributeError(reason or f'Overiding of attribute "{attribute}" not allowed')
            return super().__new__(mcs, name, bases, attrs)

    return LimitedClass


class _SubsystemView(torch.nn.Module):
    """[B, 2^n] <-> [(B * 2^(n-m)), 2^m] with `qubits` as the fast axis.
    Qubit q is axis q of the [B, 2, ..., 2] view (qubit 0 most significant)."""

    def __init__(self, num_qubits: int, qubits: typing.List[int], inverse: bool):
        super().__init__()
        self.n = num_qubits
        self.inner = list(qubits)
        self.outer = [q for q in range(num_qubits) if q not in self.inner]
        self.inverse = inverse
        order = [0] + [1 + q for q in self.outer] + [1 + q for q in self.inner]
        self.order = order
        self.back = [order.index(k) for k in range(num_qubits + 1)]

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        n, m = self.n, len(self.inner)
        if not self.inverse:
            b = x.shape[0]
            y = x.reshape([b] + [2] * n).permute(self.order)
            return y.reshape(b * (1 << (n - m)), 1 << m)
        b = x.shape[0] >> (n - m)
        y = x.reshape([b] + [2] * (n - m) + [2] * m).permute(self.back)
        return y.reshape(b, 1 << n)


def get_matrix_transforms(num_qubits: int, in_circuit: typing.List[int]
                          ) -> typing.Tuple[torch.nn.Module, torch.nn.Module]:
    """(to_matrix, to_state) modules for the subsystem `in_circuit`."""
    return _SubsystemView(num_qubits, in_circuit, False), _SubsystemView(num_qubits, in_circuit, True)

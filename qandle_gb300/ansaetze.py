"""Ansaetze (mirrors qandle/ansaetze/).

* StronglyEntanglingLayer (stronglyentangling.py): rotations on every listed
  qubit per layer, then a CNOT ring of range (layer mod (len(qubits)-1)) + 1.
* TwoLocal (twolocal.py), SpecialUnitary / SU (specialunitary.py) and
  StronglyEntanglingLayerBudget (stronglyentangling_budget.py).

Every built ansatz exposes ``applied_gates``: its gates, built, in the order
that gives the reference's forward result, so both engines (and the in-place
per-gate path) run it without a kernel of its own.  The reference's built
TwoLocal and SU apply their CNOT chain as one matrix product on a column
vector, ``(C_0 C_1 ... C_k) v``, i.e. the chain's last CNOT first;
``applied_gates`` keep that order, and ``decompose()`` returns the
reference's decomposition, which lists the chain first to last.  (Unlike the
reference, whose product needs an unbatched state, batched states work.)
The registered submodules carry the reference's names (SEL and TwoLocal
``mods``, SU and the budget ansatz ``layers``), so state_dicts saved with
either package load into the other.
"""
from __future__ import annotations

import copy
import typing

import torch

from . import config, remap, utils
from . import operators as op
from .embeddings import parse_rot

__all__ = ["StronglyEntanglingLayer", "StronglyEntanglingLayerBuilt", "TwoLocal", "TwoLocalBuilt",
           "SpecialUnitary", "SpecialUnitaryBuilt", "SU", "StronglyEntanglingLayerBudget"]

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

    @property
    def applied_gates(self) -> typing.List[torch.nn.Module]:
        return list(self.mods)

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
        return _decomposed_matrix(self, **kwargs)


def _decomposed_matrix(ansatz, **kwargs) -> torch.Tensor:
    """to_matrix of a built ansatz as the reference forms it
    (ansaetze/ansatz.py:26-33): the gates of decompose(), built on the
    ansatz's qubit count, their matrices combined by utils.reduce_dot (later
    gates multiply from the left; the result has a batch axis).  For gates
    that do not commute this is not the matrix of forward() in the row
    convention; it is kept identical to the reference's result."""
    gates = [g.build(num_qubits=ansatz.num_qubits) if hasattr(g, "build") else g for g in ansatz.decompose()]
    return utils.reduce_dot(*[g.to_matrix(**kwargs) for g in gates])


def _chain(qubits: typing.List[int]) -> typing.List[op.CNOT]:
    """CNOT(q0, q1), CNOT(q1, q2), ... along `qubits`."""
    return [op.CNOT(qubits[i], qubits[i + 1]) for i in range(len(qubits) - 1)]


def _chain_as_applied(qubits: typing.List[int], num_qubits: int) -> typing.List[torch.nn.Module]:
    """The chain as the reference's matrix product applies it: last CNOT first."""
    return [g.build(num_qubits) for g in reversed(_chain(qubits))]


class TwoLocal(op.UnbuiltOperator):
    """RY layers and a linear CNOT chain (twolocal.py:13-60)."""

    def __init__(self, qubits: typing.Union[typing.List[int], None] = None, depth: int = 1,
                 remapping: typing.Union[typing.Callable, None] = config.DEFAULT_MAPPING, q_params=None):
        self.depth = depth
        self.remapping = remapping
        self.q_params = q_params
        self.qubits = qubits

    def build(self, *args, **kwargs) -> "TwoLocalBuilt":
        return TwoLocalBuilt(num_qubits=kwargs["num_qubits"], qubits=self.qubits, depth=self.depth,
                             remapping=self.remapping, q_params=self.q_params)

    def __str__(self) -> str:
        return "TL"

    def to_qasm(self):
        return [g.to_qasm() for g in self.decompose()]

    def decompose(self) -> typing.List[op.Operator]:
        if self.qubits is None:
            raise ValueError("It is not specified on which qubits to apply the ansatz. Build the circuit to "
                             "specify or pass them explicitly as a list")
        qp = self.q_params if self.q_params is not None else torch.rand(self.depth, len(self.qubits))
        out = []
        for d in range(self.depth):
            out.extend(op.RY(qubit=w, theta=qp[d, wi]) for wi, w in enumerate(self.qubits))
            out.extend(_chain(self.qubits))
        return out


class TwoLocalBuilt(op.BuiltOperator):
    """Built TwoLocal (twolocal.py:63-123): per layer RY(q_params[d, w]) on
    every qubit w of the circuit (the reference indexes by circuit qubit; its
    RY use the default remapping), then the chain over `qubits`."""

    def __init__(self, num_qubits: int, qubits: typing.Union[typing.List[int], None], depth: int = 1,
                 remapping: typing.Union[typing.Callable, None] = config.DEFAULT_MAPPING, q_params=None):
        super().__init__()
        self.num_qubits = num_qubits
        self.depth = depth
        self.remapping = remapping
        self.qubits = qubits or list(range(num_qubits))
        if q_params is None or tuple(q_params.shape) != (depth, len(self.qubits)):
            q_params = torch.rand(depth, num_qubits)
        self.mods = torch.nn.ModuleList([
            torch.nn.Sequential(*[op.RY(qubit=w, theta=q_params[d, w]).build(num_qubits)
                                  for w in range(num_qubits)]) for d in range(depth)])
        chain = _chain_as_applied(self.qubits, num_qubits)
        applied = []
        for d in range(depth):
            applied.extend(self.mods[d])
            applied.extend(chain)
        # not registered: the RY modules are registered in mods, the chain
        # gates hold no parameters
        self.__dict__["_applied"] = applied
        self.__dict__["_chain"] = chain

    @property
    def applied_gates(self) -> typing.List[torch.nn.Module]:
        return self._applied

    def _apply(self, fn, *args, **kwargs):
        super()._apply(fn, *args, **kwargs)
        for m in self._chain:
            m._apply(fn, *args, **kwargs)
        return self

    def forward(self, state: torch.Tensor) -> torch.Tensor:
        for m in self.applied_gates:
            state = m(state)
        return state

    def __str__(self) -> str:
        return "TL"

    def to_qasm(self):
        out = []
        for d in range(self.depth):
            out.extend(g.to_qasm() for g in self.mods[d])
            out.extend(g.to_qasm() for g in _chain(self.qubits))
        return out

    def decompose(self) -> typing.List[op.Operator]:
        out = []
        for d in range(self.depth):
            out.extend(copy.deepcopy(g) for g in self.mods[d])
            out.extend(_chain(self.qubits))
        return out

    def to_matrix(self, **kwargs):
        return _decomposed_matrix(self, **kwargs)


class SpecialUnitary(op.UnbuiltOperator):
    """Hardware-efficient SU(2) 2-local circuit (specialunitary.py:11-56):
    rotation layers on `qubits` with a linear CNOT chain between them."""

    def __init__(self, qubits: typing.Union[typing.List[int], None] = None, reps: int = 1, rotations=("ry",)):
        self.qubits = qubits
        self.reps = reps
        self.rotations = [_ROT_CLASS[parse_rot(r)] for r in rotations]

    def build(self, *args, **kwargs) -> "SpecialUnitaryBuilt":
        return SpecialUnitaryBuilt(num_qubits=kwargs["num_qubits"], reps=self.reps, rotations=self.rotations,
                                   qubits=self.qubits)

    def __str__(self) -> str:
        return "SU"

    def to_qasm(self):
        return [g.to_qasm() for g in self.decompose()]

    def decompose(self) -> typing.List[op.Operator]:
        if self.qubits is None:
            raise ValueError("It is not specified on which qubits to apply the ansatz. Build the circuit to "
                             "specify or pass them explicitly as a list")
        out = [r(w) for r in self.rotations for w in self.qubits]
        for _ in range(self.reps):
            out.extend(_chain(self.qubits))
            out.extend(r(w) for r in self.rotations for w in self.qubits)
        return out


SU = SpecialUnitary


class SpecialUnitaryBuilt(op.BuiltOperator):
    """Built SpecialUnitary (specialunitary.py:59-123): blocks of every
    rotation on every qubit (per qubit in rotation order), the chain before
    every block after the first.  As in the reference, the subsystem
    transforms of qandle_gb300.utils are registered as submodules `to_matrix`
    / `to_state` (the `to_matrix` method still resolves first)."""

    def __init__(self, num_qubits: int, qubits: typing.Union[typing.List[int], None], reps: int, rotations):
        super().__init__()
        from .utils import get_matrix_transforms

        self.num_qubits = num_qubits
        self.reps = reps
        self.rotations = rotations
        self.qubits = qubits or list(range(num_qubits))
        self.to_matrix, self.to_state = get_matrix_transforms(num_qubits, self.qubits)
        self.layers = torch.nn.ModuleList([
            torch.nn.Sequential(*[r(w).build(num_qubits=num_qubits) for w in self.qubits for r in rotations])
            for _ in range(reps + 1)])
        chain = _chain_as_applied(self.qubits, num_qubits)
        applied = list(self.layers[0])
        for block in self.layers[1:]:
            applied.extend(chain)
            applied.extend(block)
        self.__dict__["_applied"] = applied  # rotations registered in layers
        self.__dict__["_chain"] = chain

    @property
    def applied_gates(self) -> typing.List[torch.nn.Module]:
        return self._applied

    def _apply(self, fn, *args, **kwargs):
        super()._apply(fn, *args, **kwargs)
        for m in self._chain:
            m._apply(fn, *args, **kwargs)
        return self

    def forward(self, state: torch.Tensor) -> torch.Tensor:
        for m in self.applied_gates:
            state = m(state)
        return state

    def __str__(self) -> str:
        return "SU"

    def to_matrix(self, **kwargs):  # (the registered transform modules do not shadow methods)
        return _decomposed_matrix(self, **kwargs)

    def to_qasm(self):
        return [g.to_qasm() for g in self.decompose()]

    def decompose(self) -> typing.List[op.Operator]:
        out = list(self.layers[0])
        for block in self.layers[1:]:
            out.extend(block)
            out.extend(_chain(self.qubits))
        return out


class StronglyEntanglingLayerBudget(op.BuiltOperator):
    """Strongly entangling layer with a parameter budget
    (stronglyentangling_budget.py:15-90): rotations cycle through
    `rotations`, one per qubit per layer, until `param_budget` rotations are
    placed; every `control_gate_spacing` layers a ring of control gates
    (CNOT or CZ) with a shifting range is inserted."""

    def __init__(self, num_qubits_total: int, qubits: typing.Union[typing.List[int], None] = None,
                 param_budget: int = 1, control_gate=op.CNOT, control_gate_spacing: int = 1,
                 rotations=("rz", "ry"), remapping: typing.Union[typing.Callable, None] = config.DEFAULT_MAPPING):
        super().__init__()
        assert control_gate in [op.CNOT, op.CZ], f"Control gate {control_gate} not supported"
        self.qubits = list(range(num_qubits_total)) if qubits is None else qubits
        self.num_qubits = num_qubits_total
        self.rots = [_ROT_CLASS[parse_rot(r)] for r in rotations]
        self.remapping = remap.none if remapping is None else remapping
        self.param_budget = param_budget
        self.control_gate = control_gate
        self.control_gate_spacing = control_gate_spacing
        self.layers_ub = self._allocate_params()
        self.layers = torch.nn.Sequential(*[g.build(num_qubits=num_qubits_total) for g in self.layers_ub])

    def _allocate_params(self) -> typing.List[op.UnbuiltOperator]:
        out = []
        placed = 0
        depth = 0
        ring = -1
        nq = len(self.qubits)
        while True:
            r = self.rots[depth % len(self.rots)]
            if depth > 0 and depth % self.control_gate_spacing == 0:
                ring = (ring + 1) % nq
                shift = ring % (nq - 1)
                for ci in range(nq):
                    out.append(self.control_gate(control=self.qubits[ci], target=self.qubits[(ci + 1 + shift) % nq]))
            depth += 1
            for w in self.qubits:
                placed += 1
                if placed > self.param_budget:
                    return out
                out.append(r(qubit=w, remapping=self.remapping))

    @property
    def applied_gates(self) -> typing.List[torch.nn.Module]:
        return list(self.layers)

    def __str__(self) -> str:
        return "SEL"

    def to_qasm(self):
        return [g.to_qasm() for g in self.layers_ub]

    def decompose(self) -> typing.List[op.UnbuiltOperator]:
        return self.layers_ub

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        return self.layers(x)

    def to_matrix(self, **kwargs):
        return _decomposed_matrix(self, **kwargs)

"""Gate layers, mirroring qandle's operator classes (qandle/operators.py).

Same class names, constructor arguments, attributes and errors as the
reference: an unbuilt gate (``RX(qubit, theta, name, remapping=...)``) is
built against a qubit count into a ``torch.nn.Module`` (``BuiltRX``) whose
``theta`` is a trainable Parameter.  Instead of a dense 2^n x 2^n matrix the
built module keeps only its 2x2 action, and ``forward`` runs one CUDA kernel
pass (qandle_gb300.plain).  ``to_matrix`` still returns the dense matrix for
inspection (it is never used on the execution path).

Row-vector convention as in the reference: ``forward(state)`` equals
``state @ to_matrix()``.
"""
from __future__ import annotations

import abc
import warnings
import typing

import torch

from . import config, errors, plain, qasm, remap

__all__ = [
    "Operator", "UnbuiltOperator", "BuiltOperator",
    "RX", "RY", "RZ", "BuiltRX", "BuiltRY", "BuiltRZ",
    "UnbuiltParametrizedOperator", "BuiltParametrizedOperator",
    "CNOT", "CZ", "SWAP", "BuiltCNOT", "BuiltCZ", "BuiltSWAP",
    "U", "BuiltU", "CustomGate", "BUILT_CLASS_RELATION",
    "Invert", "BuiltInvert", "Controlled", "BuiltControlled", "Reset", "BuiltReset",
]


class Operator(abc.ABC):
    """Everything that can be applied to a state (operators.py:35-49)."""

    named = False

    def to_qasm(self):
        """OpenQASM representation (qandle_gb300.qasm)."""
        raise NotImplementedError(f"{type(self).__name__} has no OpenQASM representation")

    @abc.abstractmethod
    def __str__(self) -> str: ...

    def __repr__(self) -> str:
        return self.__str__()


class UnbuiltOperator(Operator, abc.ABC):
    @abc.abstractmethod
    def build(self, num_qubits, **kwargs) -> "BuiltOperator": ...


class BuiltOperator(Operator, torch.nn.Module, abc.ABC):
    @abc.abstractmethod
    def forward(self, state: torch.Tensor) -> torch.Tensor: ...

    @abc.abstractmethod
    def to_matrix(self, **kwargs) -> torch.Tensor: ...


def _kron_embed(m2: torch.Tensor, qubit: int, num_qubits: int) -> torch.Tensor:
    """Dense kron(.., m2 at `qubit`, ..) in complex64 (inspection only)."""
    m = torch.eye(1, dtype=torch.complex64)
    for i in range(num_qubits):
        m = torch.kron(m, m2.to(torch.complex64) if i == qubit else torch.eye(2, dtype=torch.complex64))
    return m


def rotation_row_matrix(axis: int, theta: torch.Tensor) -> torch.Tensor:
    """Row-form 2x2 of RX/RY/RZ at t = theta/2 (operators.py:368-395 with the
    transposed buffers of :236-238); shape theta.shape + (2, 2)."""
    t = theta.to(torch.float32) / 2
    c, s = torch.cos(t).to(torch.complex64), torch.sin(t).to(torch.complex64)
    z = torch.zeros_like(c)
    if axis == 0:
        rows = [[c, -1j * s], [-1j * s, c]]
    elif axis == 1:
        rows = [[c, s], [-s, c]]
    else:
        rows = [[c - 1j * s, z], [z, c + 1j * s]]
    return torch.stack([torch.stack(r, -1) for r in rows], -2)


class U(UnbuiltOperator):
    """Fixed single-qubit gate; ``matrix`` is applied as state @ kron(.., M, ..)
    (operators.py:72-84)."""

    def __init__(self, qubit: int, matrix: torch.Tensor):
        self.qubit = qubit
        self.matrix = matrix

    def __str__(self) -> str:
        return f"U_{self.qubit}"

    def build(self, num_qubits, **kwargs) -> "BuiltU":
        return BuiltU(qubit=self.qubit, matrix=self.matrix, num_qubits=num_qubits)

    def to_qasm(self):
        return qasm.QasmRepresentation(gate_str="U", qubit=self.qubit)


class BuiltU(BuiltOperator):
    """Built fixed gate (operators.py:87-129).  Keeps the 2x2 only."""

    def __init__(self, qubit: int, matrix: torch.Tensor, num_qubits: int, self_description: str = "U"):
        super().__init__()
        self.qubit = qubit
        self.num_qubits = num_qubits
        self.description = self_description
        self.original_matrix = matrix
        m = torch.as_tensor(matrix).to(torch.complex64).reshape(2, 2).contiguous()
        self.register_buffer("_m", m, persistent=False)

    @property
    def matrix(self) -> torch.Tensor:
        return _kron_embed(self._m.cpu(), self.qubit, self.num_qubits)

    def __str__(self) -> str:
        return f"{self.description}_{self.qubit}"

    def forward(self, state: torch.Tensor) -> torch.Tensor:
        return plain.Matrix.apply(state, self._m, self.num_qubits, self.qubit)

    def to_matrix(self, **kwargs) -> torch.Tensor:
        return self.matrix

    def to_qasm(self):
        m = torch.as_tensor(self.original_matrix)
        u = f"{m[0, 0]:.2f}, {m[0, 1]:.2f}, {m[1, 0]:.2f}, {m[1, 1]:.2f}"
        definition = "gate " + self.description + "_" + str(self.qubit) + " q[" + str(self.qubit) + "] {{ " + \
            "U(" + u + ") }}"
        return qasm.QasmRepresentation(gate_str=definition, qubit=self.qubit)


CustomGate = BuiltU


class UnbuiltParametrizedOperator(UnbuiltOperator):
    """Parametrised gate before building (operators.py:150-212)."""

    def __init__(self, qubit: int, theta: typing.Union[float, torch.Tensor, None] = None,
                 name: typing.Union[str, None] = None, **kwargs):
        assert isinstance(qubit, int), "qubit must be an integer"
        assert qubit >= 0, "qubit must be >= 0"
        if isinstance(theta, (float, int)):
            theta = torch.tensor(theta, requires_grad=True, dtype=torch.float)
        remapping = kwargs.get("remapping", config.DEFAULT_MAPPING)
        if remapping is None:
            remapping = remap.none
        self.qubit = qubit
        self.name = name
        self.named = name is not None
        self.theta = theta
        self.remapping = remapping

    def __str__(self) -> str:
        # the reference's branches, kept as they are (operators.py:177-184):
        # an unnamed gate prints its (absent) name, a named one its angle
        if self.name is None:
            return f"{self.__class__.__name__}{self.qubit} ({self.name})"
        if self.theta is None:
            return f"{self.__class__.__name__}{self.qubit}"
        return f"{self.__class__.__name__}{self.qubit} ({self.remapping(self.theta).item():.2f})"

    def build(self, num_qubits, **kwargs) -> "BuiltParametrizedOperator":
        return BUILT_CLASS_RELATION[self.__class__](
            qubit=self.qubit, initialtheta=self.theta, name=self.name,
            remapping=self.remapping, num_qubits=num_qubits)

    def to_qasm(self):
        if self.named:
            return qasm.QasmRepresentation(gate_str=self.__class__.__name__.lower(), qubit=self.qubit,
                                           qasm3_inputs=self.name)
        if self.theta is None:
            raise errors.UnbuiltGateError("This gate has no parameter. Set parameter or build or set name "
                                          "before converting to OpenQASM2.")
        return qasm.QasmRepresentation(gate_str=self.__class__.__name__.lower(), qubit=self.qubit,
                                       gate_value=self.remapping(self.theta).item())


class BuiltParametrizedOperator(BuiltOperator, abc.ABC):
    """Built rotation (operators.py:215-305): theta is a Parameter, the angle
    used is remapping(theta), or the named input for named gates (which is
    not remapped, operators.py:266-271)."""

    axis = 0

    def __init__(self, qubit: int, remapping: typing.Callable, num_qubits: int,
                 initialtheta: typing.Union[torch.Tensor, None] = None,
                 name: typing.Union[str, None] = None):
        super().__init__()
        self.qubit = qubit
        if initialtheta is None:
            initialtheta = torch.rand(1)
        self.name = name
        self.named = name is not None
        self.theta = torch.nn.Parameter(initialtheta, requires_grad=True)
        self.remapping = remapping
        self.num_qubits = num_qubits
        self.unbuilt_class = BUILT_CLASS_RELATION.T[self.__class__]

    def __str__(self) -> str:
        base = f"{self.unbuilt_class.__name__}_{self.qubit}"
        if self.named:
            return f"{base} ({self.name})"
        return f"{base} ({self.remapping(self.theta).item():.2f})"

    def angle(self, **kwargs) -> torch.Tensor:
        """The angle theta of R(theta) = exp(-i theta/2 P) for this call."""
        if self.named:
            return torch.as_tensor(kwargs[self.name])
        return self.remapping(self.theta)

    def get_matrix(self, **kwargs) -> torch.Tensor:
        return rotation_row_matrix(self.axis, self.angle(**kwargs))

    def forward(self, state: torch.Tensor, **kwargs) -> torch.Tensor:
        return plain.Rotation.apply(state, self.angle(**kwargs), self.num_qubits, self.qubit,
                                    self.axis)

    def to_matrix(self, **kwargs) -> torch.Tensor:
        m2 = self.get_matrix(**kwargs).detach().cpu()
        if m2.dim() > 2:
            return torch.stack([_kron_embed(m, self.qubit, self.num_qubits) for m in m2.reshape(-1, 2, 2)])
        return _kron_embed(m2.reshape(2, 2), self.qubit, self.num_qubits)

    def to_qasm(self):
        if self.named:
            return qasm.QasmRepresentation(gate_str=self.unbuilt_class.__name__.lower(), qubit=self.qubit,
                                           qasm3_inputs=self.name)
        return qasm.QasmRepresentation(gate_str=self.unbuilt_class.__name__.lower(), qubit=self.qubit,
                                       gate_value=self.remapping(self.theta).item())


class RX(UnbuiltParametrizedOperator):
    """Parametrised RX gate (operators.py:308-325)."""


class RY(UnbuiltParametrizedOperator):
    """Parametrised RY gate (operators.py:328-345)."""


class RZ(UnbuiltParametrizedOperator):
    """Parametrised RZ gate (operators.py:348-365)."""


class BuiltRX(BuiltParametrizedOperator):
    axis = 0


class BuiltRY(BuiltParametrizedOperator):
    axis = 1


class BuiltRZ(BuiltParametrizedOperator):
    axis = 2


class CNOT(UnbuiltOperator):
    """CNOT gate (operators.py:398-413)."""

    def __init__(self, control: int, target: int):
        assert control != target, "Control and target must be different"
        self.c = control
        self.t = target

    def __str__(self) -> str:
        return f"CNOT {self.c}|{self.t}"

    def build(self, num_qubits, **kwargs) -> "BuiltCNOT":
        return BuiltCNOT(control=self.c, target=self.t, num_qubits=num_qubits)

    def to_qasm(self):
        return qasm.QasmRepresentation(gate_str=f"cx q[{self.c}], q[{self.t}]")


class CZ(UnbuiltOperator):
    """CZ gate (operators.py:518-533)."""

    def __init__(self, control: int, target: int):
        assert control != target, "Control and target must be different"
        self.c = control
        self.t = target

    def __str__(self) -> str:
        return f"CZ {self.c}|{self.t}"

    def build(self, num_qubits, **kwargs) -> "BuiltCZ":
        return BuiltCZ(control=self.c, target=self.t, num_qubits=num_qubits)

    def to_qasm(self):
        return qasm.QasmRepresentation(gate_str=f"cz q[{self.c}], q[{self.t}]")


class SWAP(UnbuiltOperator):
    """SWAP gate (operators.py:686-699)."""

    def __init__(self, a: int, b: int):
        self.a = a
        self.b = b

    def __str__(self) -> str:
        return f"Swap {self.a}|{self.b}"

    def build(self, num_qubits, **kwargs) -> "BuiltSWAP":
        return BuiltSWAP(a=self.a, b=self.b, num_qubits=num_qubits)

    def to_qasm(self):
        return qasm.QasmRepresentation(gate_str=f"swap q[{self.a}], q[{self.b}]")


def _check_wires(num_qubits: int, *qubits: int) -> None:
    """The reference forms the shift count n-1-q for every wire of a
    permutation gate when it builds it (operators.py:546-555, :580-588,
    :661-671); a wire q >= n makes the count negative and raises ValueError
    there.  Built gates here raise the same error at the same point."""
    for q in qubits:
        if q >= num_qubits:
            raise ValueError(f"negative shift count: qubit {q} of a gate on {num_qubits} qubits")


def _perm_matrix(fn, num_qubits):
    dim = 2 ** num_qubits
    m = torch.zeros(dim, dim, dtype=torch.complex64)
    for i in range(dim):
        j, sgn = fn(i)
        m[j, i] = sgn  # column i of M = where input basis state i goes (row form)
    return m


class BuiltCNOT(BuiltOperator):
    """out[i] = in[i ^ (1<<t2)] where bit c2 of i is set (operators.py:536-568)."""

    def __init__(self, control: int, target: int, num_qubits: int):
        super().__init__()
        self.c = control
        self.t = target
        self.num_qubits = num_qubits
        _check_wires(num_qubits, control, target)

    def forward(self, state: torch.Tensor) -> torch.Tensor:
        return plain.Permutation.apply(state, self.num_qubits, "cnot", self.c, self.t)

    def __str__(self) -> str:
        return f"CNOT {self.c}|{self.t}"

    def to_matrix(self, **kwargs) -> torch.Tensor:
        n = self.num_qubits
        c2, t2 = n - self.c - 1, n - self.t - 1
        return _perm_matrix(lambda i: ((i ^ (1 << t2)) if i & (1 << c2) else i, 1.0), n).T.contiguous()

    def to_qasm(self):
        return CNOT(self.c, self.t).to_qasm()


class BuiltCZ(BuiltOperator):
    """Negate amplitudes with both bits set (operators.py:570-601)."""

    def __init__(self, control: int, target: int, num_qubits: int):
        super().__init__()
        self.c = control
        self.t = target
        self.num_qubits = num_qubits
        _check_wires(num_qubits, control, target)

    def forward(self, state: torch.Tensor) -> torch.Tensor:
        return plain.Permutation.apply(state, self.num_qubits, "cz", self.c, self.t)

    def __str__(self) -> str:
        return f"CZ {self.c}|{self.t}"

    def to_matrix(self, **kwargs) -> torch.Tensor:
        n = self.num_qubits
        m = (1 << (n - self.c - 1)) | (1 << (n - self.t - 1))
        d = torch.tensor([-1.0 if (i & m) == m else 1.0 for i in range(2 ** n)], dtype=torch.complex64)
        return torch.diag(d)

    def to_qasm(self):
        return CZ(self.c, self.t).to_qasm()


class BuiltSWAP(BuiltOperator):
    """Exchange two qubits (operators.py:653-684)."""

    def __init__(self, a: int, b: int, num_qubits: int):
        super().__init__()
        self.a = a
        self.b = b
        self.num_qubits = num_qubits
        _check_wires(num_qubits, a, b)

    def forward(self, state: torch.Tensor) -> torch.Tensor:
        return plain.Permutation.apply(state, self.num_qubits, "swap", self.a, self.b)

    def __str__(self) -> str:
        return f"SWAP {self.a}|{self.b}"

    def to_matrix(self, **kwargs) -> torch.Tensor:
        n = self.num_qubits
        a2, b2 = n - self.a - 1, n - self.b - 1

        def f(i):
            if ((i >> a2) & 1) != ((i >> b2) & 1):
                return i ^ ((1 << a2) | (1 << b2)), 1.0
            return i, 1.0

        return _perm_matrix(f, n).T.contiguous()

    def to_qasm(self):
        return SWAP(self.a, self.b).to_qasm()


class Invert(UnbuiltOperator):
    """Inverse of a target operator (operators.py:416-432)."""

    def __init__(self, target: Operator):
        self.t = target

    def __str__(self) -> str:
        return f"{self.t}^-1"

    def build(self, num_qubits, **kwargs) -> "BuiltInvert":
        return BuiltInvert(target=self.t, num_qubits=num_qubits)

    def to_qasm(self):
        return qasm.QasmRepresentation(gate_str=f"{self.t}^-1")


class BuiltInvert(BuiltOperator):
    """state @ inv(target matrix) (operators.py:435-459).  Rotations run as
    the rotation by the negated angle, U as its 2x2 inverse, CNOT / CZ / SWAP
    as themselves (involutions); no 2^n x 2^n matrix is formed."""

    def __init__(self, target: Operator, num_qubits: int):
        super().__init__()
        if hasattr(target, "build"):
            warnings.warn(
                "Building target operator in Invert. If the target operator is parameterized, this might lead to "
                "different parameter initialization. Please build the target operator before inverting it.")
            target = target.build(num_qubits)
        self.target = target
        self.num_qubits = num_qubits

    def forward(self, state: torch.Tensor) -> torch.Tensor:
        t, n = self.target, self.num_qubits
        if isinstance(t, BuiltParametrizedOperator):
            return plain.Rotation.apply(state, -t.angle(), n, t.qubit, t.axis)
        if isinstance(t, BuiltU):
            return plain.Matrix.apply(state, torch.linalg.inv(t._m), n, t.qubit)
        if isinstance(t, (BuiltCNOT, BuiltCZ, BuiltSWAP)):
            return t(state)
        if isinstance(t, BuiltInvert):
            return t.target(state)
        if isinstance(t, BuiltControlled):
            return t.forward_inverse(state)
        raise NotImplementedError(f"Invert of {type(t).__name__} is not supported")

    def __str__(self) -> str:
        return Invert(self.target).__str__()

    def to_matrix(self, **kwargs) -> torch.Tensor:
        return torch.linalg.inv(self.target.to_matrix())

    def to_qasm(self):
        return Invert(self.target).to_qasm()


class Controlled(UnbuiltOperator):
    """Apply the target operator where the control qubit is 1 (operators.py:462-478)."""

    def __init__(self, control: int, target: Operator):
        self.c = control
        self.t = target

    def __str__(self) -> str:
        return f"Controlled {self.c}|{self.t}"

    def build(self, num_qubits, **kwargs) -> "BuiltControlled":
        return BuiltControlled(control=self.c, target=self.t, num_qubits=num_qubits)

    def to_qasm(self):
        return qasm.QasmRepresentation(gate_str=f"controlled q[{self.c}], {self.t}")


class BuiltControlled(BuiltOperator):
    """Target on the control-1 subspace, control-0 amplitudes kept
    (operators.py:481-515).  Rotation and U targets run on the controlled 2x2
    kernel; other targets use the reference's own construction (the target's
    full matrix on the control-1 rows) on the device, for up to 12 qubits."""

    def __init__(self, control: int, target: Operator, num_qubits: int):
        super().__init__()
        self.c = control
        if hasattr(target, "build"):
            target = target.build(num_qubits)
        self.t = target
        self.named = target.named
        self.num_qubits = num_qubits

    def forward(self, state: torch.Tensor, **kwargs) -> torch.Tensor:
        return self._run(state, False, **kwargs)

    def forward_inverse(self, state: torch.Tensor, **kwargs) -> torch.Tensor:
        return self._run(state, True, **kwargs)

    def _run(self, state, inverse: bool, **kwargs):
        t, n = self.t, self.num_qubits
        if isinstance(t, BuiltParametrizedOperator):
            a = t.angle(**kwargs)
            return plain.ControlledRotation.apply(state, -a if inverse else a, n, self.c, t.qubit, t.axis)
        if isinstance(t, BuiltU):
            m = torch.linalg.inv(t._m) if inverse else t._m
            return plain.ControlledMatrix.apply(state, m, n, self.c, t.qubit)
        if n > 12:
            raise NotImplementedError("Controlled of a multi-qubit target is limited to 12 qubits")
        m = t.to_matrix(**kwargs).to(device=state.device, dtype=torch.complex64)
        if inverse:
            m = torch.linalg.inv(m)
        mask = (torch.arange(1 << n, device=state.device) >> (n - 1 - self.c)) & 1 == 1
        st = state.unsqueeze(0) if state.dim() == 1 else state
        c1 = torch.where(mask, st, torch.zeros_like(st))
        out = torch.where(mask, torch.squeeze(c1.unsqueeze(1) @ m, 1), st)
        return out.squeeze(0) if state.dim() == 1 else out

    def __str__(self) -> str:
        return Controlled(self.c, self.t).__str__()

    def to_matrix(self, **kwargs) -> torch.Tensor:
        return self.t.to_matrix()  # what the reference returns (operators.py:514-515)

    def to_qasm(self):
        return Controlled(self.c, self.t).to_qasm()


class Reset(UnbuiltOperator):
    """Reset a qubit to |0> while preserving the norm (operators.py:632-650)."""

    def __init__(self, qubit: int):
        self.qubit = qubit

    def __str__(self) -> str:
        return f"Reset {self.qubit}"

    def build(self, num_qubits, **kwargs) -> "BuiltReset":
        return BUILT_CLASS_RELATION[self.__class__](qubit=self.qubit, num_qubits=num_qubits)

    def to_qasm(self):
        return qasm.QasmRepresentation(gate_str="reset", qubit=self.qubit)


class BuiltReset(BuiltOperator):
    """Per pair of amplitudes differing in the qubit: a0 * |pair| / (|a0| +
    1e-7) on |0>, 0 on |1> (operators.py:603-629)."""

    def __init__(self, qubit: int, num_qubits: int):
        super().__init__()
        if not 0 <= qubit < num_qubits:
            # the reference's subsystem reshape fails here (an einops
            # RuntimeError, operators.py:608-610)
            raise RuntimeError(f"Reset of qubit {qubit} in a circuit of {num_qubits} qubits")
        self.qubit = qubit
        self.num_qubits = num_qubits

    def forward(self, state: torch.Tensor) -> torch.Tensor:
        return plain.Reset.apply(state, self.num_qubits, self.qubit)

    def __str__(self) -> str:
        return Reset(self.qubit).__str__()

    def to_matrix(self, **kwargs) -> torch.Tensor:
        raise ValueError("Reset gate does not have a matrix representation.")

    def to_qasm(self):
        return Reset(self.qubit).to_qasm()


class rdict(dict):
    """Reversible dict (operators.py:702-706)."""

    @property
    def T(self):
        return {v: k for k, v in self.items()}


BUILT_CLASS_RELATION = rdict({
    UnbuiltOperator: BuiltOperator,
    UnbuiltParametrizedOperator: BuiltParametrizedOperator,
    RX: BuiltRX,
    RY: BuiltRY,
    RZ: BuiltRZ,
    CNOT: BuiltCNOT,
    U: BuiltU,
    SWAP: BuiltSWAP,
    CZ: BuiltCZ,
    Reset: BuiltReset,
})

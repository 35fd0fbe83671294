"""Circuit front end (mirrors qandle/qcircuit.py:13-212).

``Circuit(layers, num_qubits=None, ...)`` builds its layers exactly like the
reference and runs them on one of two executors:

* ``engine="fused"`` (default): the circuit is lowered once to a gate
  program and run by the fused CUDA engine (qandle_gb300.engine) -- gate
  fusion into shared-memory passes; an inference call with a measured output
  replays one captured CUDA graph of the whole forward (kept per device,
  batch and input kind); a call that needs gradients launches the passes
  and runs the adjoint backward.
* ``engine="plain"``: the reference's per-layer loop
  (UnsplittedCircuit.forward, qcircuit.py:163-174) with one CUDA kernel pass
  per gate (qandle_gb300.plain).

Both return what the reference returns for the same layers and inputs.
"""
from __future__ import annotations

import typing
import warnings

import torch

from . import operators, utils
from . import measurements

__all__ = ["Circuit", "UnsplittedCircuit", "SplittedCircuit", "Subcircuit"]


class Circuit(torch.nn.Module):
    def __init__(self, layers: typing.List[operators.Operator], num_qubits=None,
                 split_max_qubits=0, circuit=None, engine: str = "fused", **engine_options):
        super().__init__()
        self.name = ""
        self.named = True
        if not hasattr(layers, "__iter__"):
            layers = [layers]
        if num_qubits is not None:
            self.num_qubits = num_qubits
        else:
            self.num_qubits = len(self._used_qubits(layers))
        if engine not in ("fused", "plain"):
            raise ValueError(f"engine must be 'fused' or 'plain', got {engine!r}")
        self.engine = engine
        if circuit is not None:
            self.circuit = circuit
        elif split_max_qubits > 0 and self.num_qubits > split_max_qubits:
            from . import splitter

            self.circuit = SplittedCircuit(
                self.num_qubits, splitter.split(_UnbuiltLayers(self.num_qubits, layers), max_qubits=split_max_qubits))
        else:
            self.circuit = UnsplittedCircuit(self.num_qubits, layers)
        self._executor = None
        self._engine_options = engine_options

    def __getstate__(self):
        # the fused executor holds library handles, device tables and a lock;
        # a copy (copy.deepcopy, pickling, torch.save of the module) leaves it
        # out and plans again at its first call
        state = self.__dict__.copy()
        state["_executor"] = None
        return state

    def forward(self, state=None, **kwargs):
        if self.engine == "plain":
            return self.circuit.forward(state, **kwargs)
        if self._executor is None:
            from . import engine as _engine

            self._executor = _engine.FusedExecutor(self.circuit, **self._engine_options)
        return self._executor(state, **kwargs)

    def tune(self, batch: int, device="cuda", **kwargs) -> dict:
        """Pick the fused engine's plan options for this circuit at `batch`
        by timing candidates on `device` (qandle_gb300.tune.autotune; the
        answer is cached on disk) and use them from the next call on."""
        from . import tune as _tune

        res = _tune.autotune(self, batch, device, **kwargs)
        self._engine_options = dict(self._engine_options, **res["options"])
        self._executor = None
        return res

    def to_matrix(self, **kwargs):
        return self.circuit.to_matrix(**kwargs)

    def to_qasm(self):
        return self.circuit.to_qasm()

    def to_openqasm2(self) -> str:
        from . import qasm

        return qasm.convert_to_qasm(self, qasm_version=2, include_header=True)

    def to_openqasm3(self) -> str:
        from . import qasm

        return qasm.convert_to_qasm(self, qasm_version=3, include_header=True)

    @classmethod
    def from_qasm(cls, text: str, **options) -> "Circuit":
        """A circuit from OpenQASM 2/3 text in the supported subset
        (qandle_gb300.qasm.parse); named angles become named inputs."""
        from . import qasm

        layers, n = qasm.parse(text)
        return cls(layers, num_qubits=n, **options)

    def __matmul__(self, x):
        return self.forward(x)

    @staticmethod
    def _used_qubits(layers) -> typing.Set[int]:
        """qcircuit.py:69-106."""
        qubits = set()
        for layer in layers:
            if isinstance(layer, (operators.CNOT, operators.CZ)):
                qubits.add(layer.c)
                qubits.add(layer.t)
            elif isinstance(layer, operators.Controlled):
                qubits.add(layer.c)
                qubits.update(Circuit._used_qubits([layer.t]))
            elif isinstance(layer, operators.Invert):
                qubits.update(Circuit._used_qubits([layer.t]))
            elif isinstance(layer, operators.SWAP):
                qubits.add(layer.a)
                qubits.add(layer.b)
            elif hasattr(layer, "qubit"):
                qubits.add(layer.qubit)
            elif getattr(layer, "num_qubits", None) is not None:
                qubits.update(range(layer.num_qubits))
            elif getattr(layer, "qubits", None) is not None:
                qubits.update(layer.qubits)
            elif isinstance(layer, (measurements.UnbuiltMeasurement, measurements.BuiltMeasurement)):
                pass
            else:
                raise ValueError(f"Unknown layer type {type(layer)}, number of qubits could not be "
                                 "inferred. Pass :code:`num_qubits` to the circuit.")
        if len(qubits) == 0:
            raise ValueError("Number of qubits could not be inferred from layers. Please provide "
                             "num_qubits to the circuit directly.")
        return qubits

    def decompose(self):
        return Circuit(layers=[], num_qubits=self.num_qubits, circuit=self.circuit.decompose(),
                       engine=self.engine, **self._engine_options)

    def split(self, max_qubits):
        """The circuit cut into subcircuits of at most `max_qubits` qubits
        (qcircuit.py:112-122, qandle_gb300.splitter)."""
        if isinstance(self.circuit, SplittedCircuit):
            warnings.warn("Circuit already split, returning original circuit.")
            return self
        from . import splitter

        splitdict = splitter.split(self.circuit.decompose(), max_qubits=max_qubits)
        return Circuit(layers=[], num_qubits=self.num_qubits, circuit=SplittedCircuit(self.num_qubits, splitdict),
                       engine=self.engine, **self._engine_options)


class UnsplittedCircuit(torch.nn.Module):
    """Sequential executor (qcircuit.py:137-212); the plain engine's loop."""

    def __init__(self, num_qubits: int, layers: list):
        super().__init__()
        self.num_qubits = num_qubits
        state = torch.zeros(2 ** num_qubits, dtype=torch.complex64)
        state[0] = 1
        self.register_buffer("state", state, persistent=False)
        self.layers = torch.nn.ModuleList(self._build_layers(layers, num_qubits))

    @staticmethod
    def _build_layers(layers: list, num_qubits: int) -> typing.List[torch.nn.Module]:
        out = []
        for la in layers:
            out.append(la.build(num_qubits=num_qubits) if hasattr(la, "build") else la)
        return out

    def forward(self, state=None, **kwargs):
        if not torch.is_grad_enabled() and self._all_cuda(state, kwargs):
            # inference: one in-place kernel pass per gate on a single buffer
            from . import plain

            return plain.run_layers_inplace(list(self.layers), state, self.num_qubits, kwargs, self.state)
        if state is None:
            state = self.state
        for mod in self.layers:
            if mod.named:
                state = mod(state, **kwargs)
            else:
                state = mod(state)
        return state

    def _all_cuda(self, state, kwargs) -> bool:
        ts = [state if state is not None else self.state]
        ts += [v for v in kwargs.values() if isinstance(v, torch.Tensor)]
        return all(t.is_cuda for t in ts)

    def decompose(self) -> "UnsplittedCircuit":
        new_layers = []
        for layer in self.layers:
            if hasattr(layer, "decompose"):
                if isinstance(layer, Circuit):
                    new_layers.extend(layer.decompose().circuit.layers)
                else:
                    new_layers.extend(layer.decompose())
            else:
                new_layers.append(layer)
        return UnsplittedCircuit(self.num_qubits, new_layers)

    def split(self, **kwargs):
        """Subcircuits of this circuit (qcircuit.py:198-206, qandle_gb300.splitter)."""
        if self.num_qubits == 1:
            warnings.warn("Can't split circuit with only 1 qubit")
            return self
        from . import splitter

        return SplittedCircuit(self.num_qubits, splitter.split(self, **kwargs))

    def to_qasm(self):
        reps = []
        for layer in self.layers:
            if hasattr(layer, "to_qasm"):
                reps.extend(layer.to_qasm())
        return reps

    def to_matrix(self, **kwargs):
        """The layers' matrices combined by utils.reduce_dot, as the reference
        does (qcircuit.py:208-212): later layers multiply from the left and
        the result has a batch axis."""
        return utils.reduce_dot(*[mod.to_matrix(**kwargs) for mod in self.layers])


def _global_twin(mod: torch.nn.Module, to_global: typing.Dict[int, int], num_qubits: int) -> torch.nn.Module:
    """The built gate `mod` of a subcircuit, placed on the parent circuit's
    qubits; a rotation's twin shares the subcircuit gate's theta Parameter,
    so gradients and optimiser steps reach the subcircuit's parameters."""
    if isinstance(mod, operators.BuiltCNOT):
        return operators.BuiltCNOT(control=to_global[mod.c], target=to_global[mod.t], num_qubits=num_qubits)
    if isinstance(mod, operators.BuiltU):
        return operators.BuiltU(qubit=to_global[mod.qubit], matrix=mod.original_matrix, num_qubits=num_qubits,
                                self_description=mod.description)
    if isinstance(mod, operators.BuiltParametrizedOperator):
        twin = type(mod)(qubit=to_global[mod.qubit], remapping=mod.remapping, num_qubits=num_qubits,
                         initialtheta=mod.theta.detach().clone(), name=mod.name)
        twin.theta = mod.theta
        return twin
    if isinstance(mod, operators.BuiltReset):
        return operators.BuiltReset(qubit=to_global[mod.qubit], num_qubits=num_qubits)
    raise ValueError(f"{type(mod).__name__} cannot run inside a split circuit")


class Subcircuit(torch.nn.Module):
    """One subcircuit of a split circuit (qcircuit.py:271-313): its layers act
    on the subcircuit's qubits 0..m-1, `mapping` sends each parent qubit to
    its subcircuit qubit.  The reference reshapes the state so that the
    subcircuit's qubits form the fast axis and runs the small circuit; here
    the same gates run on the parent state at the parent qubits (twins that
    share the parameters), which is the same linear map."""

    def __init__(self, num_qubits_parent: int, mapping: typing.Dict[int, int], layers: list):
        super().__init__()
        self.num_qubits_parent = num_qubits_parent
        self.mapping = mapping
        self.layers = torch.nn.ModuleList(UnsplittedCircuit._build_layers(layers, num_qubits=len(mapping)))
        to_global = {v: k for k, v in mapping.items()}
        # not registered: the twins' parameters are the layers' own
        self.__dict__["twins"] = [_global_twin(m, to_global, num_qubits_parent) for m in self.layers]

    def _apply(self, fn, *args, **kwargs):
        super()._apply(fn, *args, **kwargs)
        for t in self.twins:
            t._apply(fn, *args, **kwargs)
        return self

    def forward(self, x, **kwargs):
        for mod in self.twins:
            x = mod(x, **kwargs) if mod.named else mod(x)
        return x

    def to_qasm(self):
        """Representations with the subcircuit qubits mapped back (qcircuit.py:297-313)."""
        import re

        to_global = {v: k for k, v in self.mapping.items()}
        reps = [mod.to_qasm() for mod in self.layers if hasattr(mod, "to_qasm")]
        out = []
        for r in reps:
            for rr in (r if isinstance(r, list) else [r]):
                if rr.qubit not in ("", None):
                    rr.qubit = to_global[rr.qubit]
                else:
                    rr.gate_str = re.sub(r"q\[(\d+)\]", lambda mt: f"q[{to_global[int(mt.group(1))]}]",
                                         rr.gate_str)
                out.append(rr)
        return out


class SplittedCircuit(UnsplittedCircuit):
    """A circuit cut into subcircuits by qandle_gb300.splitter (qcircuit.py:215-268).
    `subcircuits` hold the reference's structure; `layers` are all their gates
    on the parent qubits in subcircuit order, which is what the executors run
    (the fused engine as one program, the plain engine gate by gate)."""

    def __init__(self, num_qubits: int, subcircuitdict: dict):
        torch.nn.Module.__init__(self)
        self.num_qubits = num_qubits
        state = torch.zeros(2 ** num_qubits, dtype=torch.complex64)
        state[0] = 1
        self.register_buffer("state", state, persistent=False)
        self._check_qubit_order(subcircuitdict)
        self.subcircuits = torch.nn.ModuleList(
            [Subcircuit(num_qubits, subcircuitdict[i].mapping, subcircuitdict[i].layers) for i in subcircuitdict])

    @staticmethod
    def _check_qubit_order(subcircuitdict):
        for sc in subcircuitdict.values():
            keys = sorted(sc.mapping.keys())
            values = [sc.mapping[k] for k in keys]
            assert values == sorted(values), f"Mapping {sc.mapping} is not ordered."

    @property
    def layers(self) -> list:
        return [t for sc in self.subcircuits for t in sc.twins]

    def to_qasm(self):
        return [sc.to_qasm() for sc in self.subcircuits]

    def to_matrix(self, **kwargs):
        raise NotImplementedError("Can't get matrix representation of a splitted circuit.")

    def decompose(self) -> "UnsplittedCircuit":
        return UnsplittedCircuit(self.num_qubits, self.layers)


class _UnbuiltLayers:
    """The layers given to Circuit(...) before building, as the splitter sees
    them (qcircuit.py:17-26)."""

    def __init__(self, num_qubits: int, layers: list):
        self.num_qubits = num_qubits
        self.layers = layers

    def decompose(self):
        return self

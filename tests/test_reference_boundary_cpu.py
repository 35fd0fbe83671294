"""The drop-in boundary from the reference's side, on the CPU.

Circuits are built from the reference's own layer classes (qandle 0.1.8,
imported from its source tree or the baseline/_ref install, with the qw_map
stand-in), as a qandle user writes them.  The fused engine lowers them
(qandle/qcircuit.py:45-46 is the injection point) to exactly the gate records,
angles and tables of the same circuit built with this package's classes; the
planned program, executed by the CPU op emulator, reproduces the reference's
own torch forward; and the per-circuit binding a qandle maintainer adds
(the reference's Circuit.forward replaced by the fused executor) routes
calls into the engine."""
import os

import numpy as np
import pytest
import torch

from oracle import reference_torch as rt
from qandle_gb300 import engine, workloads
from tests import program_emulator as emu
from tests.test_planner import _runtime

SRC = "/root/reference/src"


@pytest.fixture(scope="module")
def qandle():
    path = SRC if os.path.isdir(os.path.join(SRC, "qandle")) else rt.REF_DIR
    why = rt.unavailable_reason(path)
    if why:
        pytest.skip(why)
    return rt.import_reference(path)


def _descs():
    """Small instances of the four workload families (p0 instead of <Z>:
    the reference measures P(0) per qubit)."""
    out = {
        "config1_plain": workloads.plain_small(n=8, batch=4, layers=2),
        "config2_sel": workloads.sel_reupload(n=7, batch=3, layers=3, reupload_every=2, measure="p0"),
        "config3_brick": workloads.adjoint_brick(n=6, batch=2, layers=4),
        "config4_deep": workloads.deep_u(n=6, batch=1, layers=3),
    }
    out["config3_brick"]["measure"] = "p0"
    return out


@pytest.mark.parametrize("name", sorted(_descs()))
def test_reference_circuit_lowers_like_ours(qandle, name):
    desc = _descs()[name]
    ref = engine.lower(rt.build_circuit(qandle, desc).circuit)
    ours = engine.lower(workloads.build_circuit(desc).circuit)
    assert ref.n == ours.n and ref.measure == ours.measure
    assert ref.gates == ours.gates
    assert ref.qlist == ours.qlist and ref.named_cols == ours.named_cols
    assert len(ref.umats) == len(ours.umats)
    for a, b in zip(ref.umats, ours.umats):
        assert torch.equal(a, b)
    pa = engine._gather_params(ref, "cpu") if ref.param_mods else torch.zeros(0)
    pb = engine._gather_params(ours, "cpu") if ours.param_mods else torch.zeros(0)
    assert torch.equal(pa, pb)
    ta = engine.Program(ref, ref.measure, keep_state=True, segments=2)
    tb = engine.Program(ours, ours.measure, keep_state=True, segments=2)
    assert ta.summary() == tb.summary()
    assert torch.equal(ta._table_host, tb._table_host)


@pytest.mark.parametrize("name", sorted(_descs()))
def test_reference_circuit_plan_reproduces_reference_forward(qandle, name):
    desc = _descs()[name]
    rc = rt.build_circuit(qandle, desc)
    n, B = desc["n"], desc["batch"]
    st0 = None
    if not desc["inputs"]:  # batched |0..0> so every sample has a row
        st0 = torch.zeros(B, 1 << n, dtype=torch.complex64)
        st0[:, 0] = 1
    with torch.no_grad():
        want = (rc(st0) if st0 is not None else rc(**rt.inputs(desc))).numpy()
    ex = engine.FusedExecutor(rc.circuit)
    assert ex.fusible
    lo = ex.lowered
    prog = ex.program(False)
    params, named, umats, embed = _runtime(lo, desc, B)
    st, _ = emu.run_forward(prog, n, B, params, named, umats, embed=embed,
                            state=None if st0 is None else st0.numpy().astype(complex))
    if lo.measure == "probs":
        got = np.abs(st) ** 2
    else:
        from oracle import oracle

        got = oracle.measure_p0(st)
    assert got.shape == want.shape
    assert np.abs(got - want).max() < 1e-5


def test_integration_snippet_routes_into_the_executor(qandle):
    """The per-circuit binding: the reference's Circuit keeps its object and
    its forward now runs the fused executor (on a CPU tensor the executor
    refuses loudly instead of falling back to the reference's loop)."""
    desc = workloads.sel_reupload(n=8, batch=2, layers=2, reupload_every=1, measure="p0")
    circ = rt.build_circuit(qandle, desc)
    fused = engine.FusedExecutor(circ.circuit)
    circ.circuit.forward = lambda state=None, **kw: fused(state, **kw)
    with pytest.raises(RuntimeError, match="CUDA tensors only"):
        circ(**rt.inputs(desc))

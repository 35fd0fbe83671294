"""Bounded waits of the pass kernels: the workspace status word reads QG_OK
after normal forwards / backwards, and a wait that runs out on purpose (an
mbarrier nothing completes, 1 ms limit) reports QG_ETIMEOUT without
breaking the context."""
import pytest
import torch

from qandle_gb300 import _lib, engine, workloads

pytestmark = pytest.mark.gpu

QG_ETIMEOUT = 3


def _forward(batch=4, n=14):
    desc = workloads.sel_reupload(n=n, batch=batch, layers=2, reupload_every=2)
    circ = workloads.build_circuit(desc, engine="fused").to("cuda")
    kw = workloads.circuit_inputs(desc, torch.device("cuda"))
    ex = engine.FusedExecutor(circ.circuit)
    bound = engine.BoundForward(ex, batch, "cuda")
    bound.set_inputs(**kw)
    bound.launch()
    return bound


def test_status_ok_after_forward():
    bound = _forward()
    engine.check_status(bound.ws)  # raises on a reported timeout
    assert _lib.load().qg_workspace_status(bound.ws.data_ptr(), _lib.stream()) == 0


def test_wait_timeout_is_reported_and_context_survives():
    lib = _lib.load()
    assert lib.qg_selftest_wait_timeout(1_000_000, _lib.stream()) == QG_ETIMEOUT
    # the device keeps working: a forward afterwards completes with a clean status
    bound = _forward()
    engine.check_status(bound.ws)
    out = bound.result()
    assert torch.isfinite(out).all()


def test_selftest_rejects_bad_limits():
    lib = _lib.load()
    assert lib.qg_selftest_wait_timeout(0, _lib.stream()) == 1  # QG_EINVAL
    assert lib.qg_selftest_wait_timeout(3_000_000_000, _lib.stream()) == 1

"""Serving-loop host logic on the CPU: QASM requests lower like the
description they were exported from, and a request's HBM need counts its
state, program workspace and output (no GPU needed: planning is host-only)."""
import numpy as np

from qandle_gb300 import _lib, serve, workloads
from qandle_gb300.engine import Program


def test_request_need_counts_state_workspace_and_output():
    rng = np.random.default_rng(5)
    desc = workloads.random_sel_request(rng, n_range=(12, 12), depth_range=(3, 3), batch_max=32)
    req = serve.Request(desc)
    req.lowered = serve.lower_description(desc)
    lo = req.lowered[0]
    req.prog = Program(lo, lo.measure, keep_state=False)
    need = serve.Server._device_bytes(req)
    B = desc["batch"]
    ws = _lib.load().qg_program_workspace_bytes(req.prog.handle, B, 0)
    assert ws > 0
    assert need >= (1 << 12) * 8 * B + ws + B * 12 * 4


def test_qasm_request_lowers_like_its_description():
    desc = workloads.sel_reupload(n=7, batch=3, layers=2, reupload_every=1)
    text = workloads.build_circuit(desc).to_openqasm3()
    x = desc["inputs"]["x"]
    inputs = {}
    for line in text.splitlines():
        if line.startswith("input float "):
            name = line[len("input float "):-1]
            col = int(name[2:]) if name.startswith("up") else int(name.rsplit("_", 1)[1])
            inputs[name] = x[:, col]
    req = serve.description_from_qasm(text, inputs, batch=3)
    lo_q, params_q, named_q, _ = serve.lower_description(req)
    assert lo_q.n == 7 and lo_q.measure == "z"
    # rotations, CNOTs and angle values in the exported order
    from oracle import oracle

    assert np.abs(oracle.forward(req) - oracle.forward(desc)).max() < 1e-12

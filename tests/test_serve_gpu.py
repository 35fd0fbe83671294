"""Continuous-batching serving loop: every request's result equals the oracle,
and is bit-identical whether it ran alone or mixed with other requests of
other widths; oversize requests are refused; a tight budget queues work
instead of failing."""
import numpy as np
import pytest
import torch

from oracle import oracle
from qandle_gb300 import serve, workloads

pytestmark = pytest.mark.gpu


def _requests(count=12, seed=11, n_range=(4, 14), depth_range=(2, 6), batch_max=64):
    rng = np.random.default_rng(seed)
    return [workloads.random_sel_request(rng, n_range=n_range, depth_range=depth_range, batch_max=batch_max)
            for _ in range(count)]


def test_mix_equals_alone_and_oracle(cuda_device):
    reqs = _requests()
    srv = serve.Server(cuda_device, hbm_budget=8 << 30)
    try:
        mixed = [srv.submit(d) for d in reqs]
        mixed_out = [r.future.result(timeout=120) for r in mixed]
        alone_out = []
        for d in reqs:
            r = srv.submit(d)
            alone_out.append(r.future.result(timeout=120))
    finally:
        srv.close()
    assert srv.steps > 0
    for d, a, b in zip(reqs, mixed_out, alone_out):
        assert torch.equal(a, b), d["n"]
        ref = oracle.forward(d)
        assert np.abs(a.numpy() - ref).max() < 1e-5, (d["n"], d["batch"])


def test_budget_refuses_and_queues(cuda_device):
    rng = np.random.default_rng(3)
    big = workloads.random_sel_request(rng, n_range=(14, 14), depth_range=(2, 2), batch_max=1)
    big["batch"] = 64
    big["inputs"]["x"] = np.resize(big["inputs"]["x"], (64, 14)).astype(np.float32)
    srv = serve.Server(cuda_device, hbm_budget=1 << 40)
    # room for one such request at a time: its state, workspace and output
    probe = serve.Request(big)
    probe.lowered = serve.lower_description(big)
    probe.prog = srv._program(probe.lowered[0])
    need = serve.Server._device_bytes(probe)
    assert need > (1 << 14) * 8 * 64  # more than the state alone
    srv.budget = need
    try:
        too_big = dict(big)
        too_big["batch"] = 65
        too_big["inputs"] = {"x": np.resize(big["inputs"]["x"], (65, 14)).astype(np.float32)}
        r = srv.submit(too_big)
        with pytest.raises(MemoryError):
            r.future.result(timeout=10)
        rs = [srv.submit(big) for _ in range(4)]  # queued one after another
        outs = [x.future.result(timeout=120) for x in rs]
    finally:
        srv.close()
    ref = oracle.forward(big)
    for o in outs:
        assert np.abs(o.numpy() - ref).max() < 1e-5


def test_policies_give_identical_results(cuda_device):
    """Shortest-remaining-work scheduling (the default) and oldest-first
    scheduling of every request each step run each request's tiles with the
    same kernel in the same order: their results are bit-identical."""
    reqs = _requests(count=10, seed=5)
    outs = {}
    for policy in ("srpt", "all"):
        srv = serve.Server(cuda_device, hbm_budget=8 << 30, policy=policy, step_tiles=64)
        try:
            hs = [srv.submit(d) for d in reqs]
            outs[policy] = [h.future.result(timeout=120) for h in hs]
        finally:
            srv.close()
        assert srv.steps > 0
    for d, a, b in zip(reqs, outs["srpt"], outs["all"]):
        assert torch.equal(a, b), d["n"]


def test_compiled_requests_match_oracle_and_interpreted(cuda_device):
    """Requests whose programs have been compiled run as launches of their
    compiled pass kernels: results within 1e-5 of the oracle and
    bit-identical to the interpreted multi-job kernel's (same op list, same
    arithmetic), so a request that switches between the two at a pass
    boundary gets the same bits."""
    import time

    reqs = _requests(count=6, seed=21, n_range=(10, 14), depth_range=(2, 4), batch_max=16)
    srv = serve.Server(cuda_device, hbm_budget=8 << 30, compile_min_tiles=1)
    try:
        first = [srv.submit(d) for d in reqs]
        first_out = [r.future.result(timeout=300) for r in first]
        t0 = time.time()
        while srv.compiled_programs + len(srv.compile_errors) < len(srv.programs) and time.time() - t0 < 300:
            time.sleep(0.05)
        assert not srv.compile_errors, srv.compile_errors
        assert srv.compiled_programs == len(srv.programs)
        before = srv.compiled_launches
        again = [srv.submit(d) for d in reqs]
        again_out = [r.future.result(timeout=300) for r in again]
    finally:
        srv.close()
    assert srv.compiled_launches - before == sum(r.prog.info.forward_passes for r in again)
    plain = serve.Server(cuda_device, hbm_budget=8 << 30, compile_min_tiles=None)
    try:
        interp_out = [plain.submit(d).future.result(timeout=300) for d in reqs]
    finally:
        plain.close()
    assert plain.compiled_launches == 0
    for d, a, b, c in zip(reqs, first_out, again_out, interp_out):
        ref = oracle.forward(d)
        assert np.abs(b.numpy() - ref).max() < 1e-5, (d["n"], d["batch"])
        assert np.abs(a.numpy() - ref).max() < 1e-5, (d["n"], d["batch"])
        assert torch.equal(b, c), (d["n"], d["batch"])
        assert torch.equal(a, c), (d["n"], d["batch"])


def test_prepare_compiles_before_traffic(cuda_device):
    """Server.prepare plans and compiles a structure before its requests
    arrive: every pass of a later request of that structure (at or above
    compile_min_tiles) is a compiled launch, and the result is the oracle's."""
    rng = np.random.default_rng(4)
    desc = workloads.random_sel_request(rng, n_range=(12, 12), depth_range=(3, 3), batch_max=8)
    srv = serve.Server(cuda_device, hbm_budget=8 << 30, compile_min_tiles=1)
    try:
        prog = srv.prepare(desc)
        assert prog.compiled(cuda_device) and srv.compiled_programs == 1
        out = srv.submit(desc).future.result(timeout=120)
    finally:
        srv.close()
    assert srv.compiled_launches == prog.info.forward_passes
    assert np.abs(out.numpy() - oracle.forward(desc)).max() < 1e-5


def test_compiled_job_launch_refuses_uncompiled_program(cuda_device):
    """qg_job_run_pass_compiled launches nothing and returns QG_EINVAL for a
    program whose pass kernels are not compiled on the device."""
    import ctypes

    from qandle_gb300 import _lib

    rng = np.random.default_rng(6)
    desc = workloads.random_sel_request(rng, n_range=(10, 10), depth_range=(2, 2), batch_max=2)
    lo, params, named, _ = serve.lower_description(desc)
    prog = serve.Program(lo, lo.measure, keep_state=False, tile_bits=13, low_bits=6)
    assert not prog.compiled(cuda_device)
    B = desc["batch"] or 1
    ws = prog.workspace(B, False, cuda_device)
    state = torch.zeros(B, 1 << lo.n, dtype=torch.complex64, device=cuda_device)
    out = torch.zeros(B, lo.n, dtype=torch.float32, device=cuda_device)
    job = _lib.Job(prog.handle, prog.table(cuda_device).data_ptr(), ws.data_ptr(), ws.numel(), state.data_ptr(), B,
                   0, 0, out.data_ptr())
    lib = _lib.load()
    assert lib.qg_job_run_pass_compiled(ctypes.byref(job), _lib.stream()) == 1
    assert b"not compiled" in lib.qg_last_error()

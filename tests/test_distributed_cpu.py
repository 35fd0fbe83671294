"""Data-parallel host logic with two gloo ranks on the CPU: batch shards
cover the batch exactly once, and the per-rank gradients of a mean loss,
weighted by batch share and summed by allreduce_gradients, equal the
full-batch gradient.  The per-rank gradients come from the complex128 oracle
(the checker), standing in for the GPU engine that a CPU host cannot run."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from qandle_gb300 import distributed as qd
from qandle_gb300 import workloads


def test_shard_ranges_partition_the_batch():
    for batch in (0, 1, 5, 7, 256, 1023):
        for world in (1, 2, 3, 8):
            covered = []
            for r in range(world):
                a, b = qd.shard_range(batch, r, world)
                assert 0 <= a <= b <= batch
                covered.extend(range(a, b))
            assert covered == list(range(batch))
    with pytest.raises(ValueError):
        qd.shard_range(4, 2, 2)


def _loss_grad(desc, targets):
    """Mean-squared <Z> loss over the given samples: dtheta from the oracle."""
    from oracle import oracle
    st = oracle.run(desc)
    z = oracle.measure(dict(desc, measure="z"), st)
    _, dp0 = oracle.mse_z_grad(z, targets)
    dth, _, _ = oracle.adjoint(dict(desc, measure="p0"), dp0, "p0")
    return dth


def _slice_desc(desc, a, b):
    d = dict(desc)
    d["batch"] = b - a
    d["inputs"] = {k: np.asarray(v)[a:b] for k, v in desc["inputs"].items()}
    return d


def _worker(rank, world, port, desc, targets, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        a, b = qd.shard_range(desc["batch"], rank, world)
        # the oracle's loss is a mean over its own samples: undo it, the
        # weight below applies the global mean
        g = _loss_grad(_slice_desc(desc, a, b), targets[a:b]) * ((b - a) / 1.0)
        p = torch.nn.Parameter(torch.zeros(g.shape[0], dtype=torch.float32))
        p.grad = torch.tensor(g, dtype=torch.float32)
        qd.allreduce_gradients([p], weight=1.0 / desc["batch"])
        out[rank] = p.grad.numpy().copy()
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_gradient_allreduce_equals_full_batch():
    desc = workloads.sel_reupload(n=6, batch=7, layers=2, reupload_every=1, measure="z")
    rng = np.random.default_rng(5)
    targets = rng.uniform(-1, 1, size=(7, 6))
    full = _loss_grad(desc, targets)
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, desc, targets, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        got = [out[0], out[1]]
    assert np.allclose(got[0], got[1])
    assert np.abs(got[0] - full).max() < 1e-5 * max(1.0, np.abs(full).max())


def test_allreduce_keeps_float64_precision():
    # one process, no process group: the flat buffer still round-trips the
    # gradients, and a float64 gradient keeps digits float32 would drop
    p64 = torch.nn.Parameter(torch.zeros(3, dtype=torch.float64))
    p32 = torch.nn.Parameter(torch.zeros(2, dtype=torch.float32))
    p64.grad = torch.tensor([1.0 + 1e-12, -2.0, 3.0], dtype=torch.float64)
    p32.grad = torch.tensor([0.5, 0.25], dtype=torch.float32)
    qd.allreduce_gradients([p64, p32], weight=1.0)
    assert p64.grad.dtype == torch.float64
    assert p64.grad[0].item() == 1.0 + 1e-12
    assert torch.equal(p32.grad, torch.tensor([0.5, 0.25]))

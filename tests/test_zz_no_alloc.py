"""qg_measure_p0_noalloc: P0 for callers that cannot allocate device memory
when they measure (graph-captured code that must not add allocation nodes,
real-time loops, hosts whose allocator owns all device memory).

It is called through the C ABI and must equal qg_measure_p0 (which takes a
caller-provided scratch buffer) on two calls in a row -- the second call
reuses the static array the first one left behind.  This file is collected
last so that a failure here stops a run only after every other test ran; it
also passes alone in a fresh process (the first call on the device does the
one-time address look-up)."""
import ctypes

import numpy as np
import pytest
import torch

from qandle_gb300 import _lib

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _p0_with_scratch(st, n):
    lib = _lib.load()
    B = st.shape[0]
    out = torch.empty(B, n, dtype=torch.float32, device=st.device)
    scr = torch.empty(max(16, lib.qg_measure_p0_scratch_bytes(B, n)), dtype=torch.uint8, device=st.device)
    _lib.call("qg_measure_p0", st.data_ptr(), out.data_ptr(), B, n, scr.data_ptr(), scr.numel(), _lib.stream())
    return out


def _p0_noalloc(st, n):
    B = st.shape[0]
    out = torch.empty(B, n, dtype=torch.float32, device=st.device)
    _lib.call("qg_measure_p0_noalloc", st.data_ptr(), out.data_ptr(), B, n, _lib.stream())
    return out


@pytest.mark.parametrize("n,batch", [(14, 3), (5, 40)])
def test_noalloc_equals_scratch_version_twice(cuda_device, n, batch):
    g = torch.Generator().manual_seed(n)
    outs = []
    for call in range(2):
        st = torch.randn(batch, 1 << n, generator=g, dtype=torch.complex64)
        st = (st / st.abs().pow(2).sum(-1, keepdim=True).sqrt()).to(cuda_device)
        ref = _p0_with_scratch(st, n)
        got = _p0_noalloc(st, n)
        torch.cuda.synchronize()
        assert np.abs(got.cpu().numpy() - ref.cpu().numpy()).max() < TOL, call
        outs.append(got.cpu())
    assert not torch.equal(outs[0], outs[1])  # two different inputs, no stale result


def test_noalloc_refuses_oversize(cuda_device):
    lib = _lib.load()
    st = torch.zeros(1, 1 << 5, dtype=torch.complex64, device=cuda_device)
    out = torch.empty(1, 5, dtype=torch.float32, device=cuda_device)
    # 2^20 qubit-chunk partials at n = 20 need batch * 256 * 13 floats; this
    # batch asks for more than the static array holds (checked before launch)
    rc = lib.qg_measure_p0_noalloc(ctypes.c_void_p(st.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                   400, 20, None)
    assert rc == 4
    assert b"static array" in lib.qg_last_error()
    # a batch so large that batch * partials-per-sample wraps int64 is refused too
    rc = lib.qg_measure_p0_noalloc(ctypes.c_void_p(st.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                   1 << 62, 20, None)
    assert rc == 4
    assert b"static array" in lib.qg_last_error()

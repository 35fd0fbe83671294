"""Compiled forward passes on the host: the generated source unrolls every op
of its pass, and every pass of the benchmark-scale programs builds for
sm_103a with NVRTC (compile only; no GPU needed)."""
import pytest

from qandle_gb300 import _lib, engine, workloads


def _program(desc, **opts):
    circ = workloads.build_circuit(desc, engine="plain")
    lo = engine.lower(circ.circuit)
    return engine.Program(lo, lo.measure, keep_state=False, **opts)


def _nvrtc_or_skip(prog):
    try:
        prog.compile(load=False)
    except RuntimeError as e:
        if "libnvrtc" in str(e):
            pytest.skip("NVRTC is not installed")
        raise


def test_source_unrolls_every_op():
    prog = _program(workloads.sel_reupload(n=14, batch=2, layers=3, reupload_every=2))
    for p, pd in enumerate(prog.passes()):
        src = prog.pass_source(p)
        body = src[src.index("static void apply"):src.index("\n};")]
        skip = ("const float4* staged", "(void)staged;")
        skip = skip + ("int swb", "(void)swb;")
        calls = [ln for ln in body.splitlines()[1:]
                 if (ln.strip().endswith(";") or ln.strip().startswith("{ cta_sync<"))
                 and not ln.strip().startswith(skip)]
        assert len(calls) == len(pd["ops"]), p
        assert "switch" not in src and "qg_fwd_pass" in src
    with pytest.raises(IndexError):
        prog.pass_source(prog.info.forward_passes)


@pytest.mark.parametrize("name,opts", [
    ("sel_reupload", {}),
    ("sel_reupload", dict(tile_bits=12, reg_bits=4)),
    ("adjoint_brick", dict(tile_bits=11, low_bits=5, max_high=1)),
    ("deep_u", {}),
    ("plain_small", {}),
])
def test_compiles_for_sm103a(name, opts):
    desc = getattr(workloads, name)()
    if name == "deep_u":
        desc = workloads.deep_u(n=16, batch=1, layers=4)
    prog = _program(desc, **opts)
    _nvrtc_or_skip(prog)


def test_compile_reports_errors_through_status():
    lib = _lib.load()
    assert lib.qg_program_compile(None, 1) == 1  # QG_EINVAL
    assert b"null" in lib.qg_last_error()


def test_pending_x_ops_compile_forward_and_backward():
    """OP_XMAT (a register's pending X applied before an exchange whose
    writes it would bank-conflict) unrolls into jmaterialize in the forward
    and jmaterialize2 (psi and lambda) in the backward, and both build."""
    desc = workloads.adjoint_brick(n=15, batch=1, layers=6)
    desc["measure"] = "p0"
    lo = engine.lower(workloads.build_circuit(desc, engine="plain").circuit)
    prog = engine.Program(lo, "p0", keep_state=True, segments=2)
    fwd = [p for p, pd in enumerate(prog.passes()) if (pd["ops"][:, 0] == 8).any()]
    bwd = [p for p, pd in enumerate(prog.passes(True)) if (pd["ops"][:, 0] == 8).any()]
    assert fwd and bwd
    assert "jmaterialize<" in prog.pass_source(fwd[0])
    assert "jmaterialize2<" in prog.pass_source(bwd[0], backward=True)
    try:
        prog.compile(load=False, backward=True)
    except RuntimeError as e:
        if "libnvrtc" in str(e):
            pytest.skip("NVRTC is not installed")
        raise

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

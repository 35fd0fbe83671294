"""The C-ABI library builds, loads without a GPU and exports every symbol the
public header declares (no compute calls: this runs on CPU)."""
import os
import re

import pytest

from qandle_gb300 import _lib, build

HEADERS = [os.path.join(build.INCLUDE, f) for f in os.listdir(build.INCLUDE) if f.endswith(".h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        with open(h) as f:
            text = f.read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(qg_\w+)\s*\(", text))
    return sorted(names)


def test_header_declares_symbols():
    assert len(declared_symbols()) >= 10


def test_library_exports_all_declared_symbols():
    lib = _lib.load()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # every symbol the ctypes layer binds is declared in the header
    assert set(_lib.SIGNATURES) <= set(declared_symbols())


def test_version_and_error_reporting():
    lib = _lib.load()
    assert lib.qg_version() >= 100
    # an invalid argument is rejected on the host before any CUDA call
    rc = lib.qg_apply_cnot(None, 1, 3, 0, 1, None)
    assert rc == 1
    assert b"state is null" in lib.qg_last_error()
    with pytest.raises(RuntimeError, match="out of range"):
        _lib.call("qg_apply_cz", 16, 1, 3, 0, 7, None)


def test_job_entry_points_refuse_bad_arguments_on_the_host():
    """The multi-job and compiled-job pass launches reject a null job list /
    job and an out-of-range job count before any CUDA call."""
    lib = _lib.load()
    assert lib.qg_job_run_pass_compiled(None, None) == 1
    assert b"job is null" in lib.qg_last_error()
    assert lib.qg_jobs_run_pass(None, 33, None) == 1
    assert lib.qg_jobs_run_pass(None, 1, None) == 1
    assert lib.qg_jobs_run_pass(None, 0, None) == 0  # nothing to launch

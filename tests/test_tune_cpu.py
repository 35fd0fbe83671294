"""Autotuner host logic: the structure key ignores angles but not gates or
qubits, the fastest candidate wins, rejected candidates are skipped, and the
answer is served from the JSON cache afterwards (timings are injected: no
GPU is needed)."""
import json

import pytest

from qandle_gb300 import engine, tune, workloads


def _circuit(desc):
    return workloads.build_circuit(desc, engine="fused")


def _load(path):
    with open(path) as f:
        return json.load(f)


def test_structure_key_ignores_angles_only():
    a = workloads.sel_reupload(n=8, batch=4, layers=2, reupload_every=1)
    b = workloads.sel_reupload(n=8, batch=4, layers=2, reupload_every=1)
    b["gates"] = [(g[0], g[1], g[2] + 0.5, g[3]) if g[0] in ("rx", "ry", "rz") and g[3] is None else g
                  for g in b["gates"]]
    c = workloads.sel_reupload(n=8, batch=4, layers=3, reupload_every=1)
    ka, kb, kc = (tune.structure_key(engine.lower(_circuit(d).circuit)) for d in (a, b, c))
    assert ka == kb and ka != kc


def test_autotune_picks_fastest_and_caches(tmp_path):
    circ = _circuit(workloads.sel_reupload(n=10, batch=4, layers=2, reupload_every=1))
    cache = str(tmp_path / "tune.json")
    cands = [dict(tile_bits=13, low_bits=6), dict(tile_bits=12, low_bits=6), dict(tile_bits=11, low_bits=5)]
    speed = {13: 3.0, 12: 1.5, 11: 2.0}
    calls = []

    def timer(opt):
        calls.append(opt)
        if opt["tile_bits"] == 11:
            raise RuntimeError("planner rejected this shape")
        return speed[opt["tile_bits"]]

    res = tune.autotune(circ, 4, "cpu", candidates=cands, cache_path=cache, timer=timer)
    assert res["options"] == dict(tile_bits=12, low_bits=6) and res["ms"] == 1.5 and not res["cached"]
    assert len(res["timings"]) == 2 and len(calls) == 3
    stored = _load(cache)
    assert len(stored) == 1
    again = tune.autotune(circ, 4, "cpu", candidates=cands, cache_path=cache, timer=timer)
    assert again["cached"] and again["options"] == res["options"] and len(calls) == 3
    other = tune.autotune(circ, 8, "cpu", candidates=cands, cache_path=cache, timer=timer)
    assert not other["cached"] and len(_load(cache)) == 2


def test_autotune_needs_a_runnable_candidate(tmp_path):
    circ = _circuit(workloads.sel_reupload(n=10, batch=4, layers=1, reupload_every=1))

    def timer(opt):
        raise RuntimeError("no")

    with pytest.raises(RuntimeError):
        tune.autotune(circ, 4, "cpu", candidates=[dict(tile_bits=13)], cache_path=str(tmp_path / "t.json"),
                      timer=timer)

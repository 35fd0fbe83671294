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


def test_staged_search_tries_k_and_remap_schedule(tmp_path):
    """Without a candidate list the search runs the tile shapes, then k one
    and two below the tile's strided limit on the best shape, then the
    searched remap schedule on the best so far, then pass lengths of 16 and
    32 2x2 slots and uncapped passes."""
    circ = _circuit(workloads.sel_reupload(n=16, batch=4, layers=2, reupload_every=1))
    calls = []

    def timer(opt):
        calls.append(dict(opt))
        ms = 2.0 if opt["tile_bits"] == 12 else 3.0
        if opt.get("max_high") == 5:  # tile 12, low 6: limit 6, so k = 5 and 4 are tried
            ms -= 0.5
        if opt.get("reg_search"):
            ms -= 0.25
        return ms

    res = tune.autotune(circ, 4, "cpu", cache_path=str(tmp_path / "t.json"), timer=timer)
    assert calls[:len(tune.DEFAULT_CANDIDATES)] == tune.DEFAULT_CANDIDATES
    ks = [c.get("max_high") for c in calls if "max_high" in c and not c.get("reg_search")]
    assert ks == [5, 4]
    rs = [c for c in calls if c.get("reg_search")]
    assert rs[0].get("max_high") == 5 and "fwd_max_mats" not in rs[0]
    assert [c.get("fwd_max_mats") for c in calls[-3:]] == [16, 32, tune.UNCAPPED]
    assert all(c.get("reg_search") == 1 and c.get("max_high") == 5 for c in calls[-3:])
    assert res["options"] == rs[0] and res["ms"] == 1.25

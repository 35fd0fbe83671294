"""Checkpoint compatibility with the reference: the state_dict keys, shapes
and dtypes and the parameter names of circuits, ansaetze, special gates,
embeddings, split and nested circuits and QConv equal the reference's
(tests/golden/state_dicts.npz, made by running qandle on the same modules;
tests/golden/make_golden.py:state_dict_modules builds them for either
package), so a checkpoint saved with qandle loads into qandle_gb300 with
strict=True, and the loaded values are the ones the module then uses."""
import json

import pytest
import torch

import qandle_gb300 as q
from tests.golden import make_golden as mg
from tests import golden_io

GOLDEN = golden_io.load("state_dicts")


def _ours():
    saved = q.config.DEFAULT_MAPPING
    q.config.DEFAULT_MAPPING = q.remap.none
    try:
        return mg.state_dict_modules(q)
    finally:
        q.config.DEFAULT_MAPPING = saved


MODS = _ours()


@pytest.mark.parametrize("name", sorted(GOLDEN.files))
def test_state_dict_layout_matches_reference(name):
    rec = json.loads(str(GOLDEN[name]))
    mod = MODS[name]
    got = [[k, list(v.shape), str(v.dtype)] for k, v in mod.state_dict().items()]
    assert got == rec["state_dict"]
    assert [k for k, _ in mod.named_parameters()] == rec["parameters"]


@pytest.mark.parametrize("name", sorted(GOLDEN.files))
def test_reference_checkpoint_loads_strictly(name):
    """A state_dict with the reference's keys and shapes (values made up
    here) loads with strict=True and lands in the parameters the module
    runs with."""
    rec = json.loads(str(GOLDEN[name]))
    mod = MODS[name]
    g = torch.Generator().manual_seed(0)
    sd = {}
    for k, shape, dtype in rec["state_dict"]:
        dt = getattr(torch, dtype.split(".")[-1])
        v = torch.randn(shape, generator=g)
        sd[k] = v.to(dt) if not dt.is_complex else torch.complex(v, v).to(dt)
    mod.load_state_dict(sd, strict=True)
    params = dict(mod.named_parameters())
    for k in rec["parameters"]:
        assert torch.equal(params[k].detach(), sd[k])


def test_twolocal_runs_the_loaded_angles():
    """TwoLocal keeps the reference's `mods` (one Sequential of RY per
    layer); the gates it runs are those modules, so loaded angles are used."""
    mod = MODS["twolocal"].circuit.layers[0]
    ry = [m for m in mod.applied_gates if hasattr(m, "theta")]
    assert [id(m) for m in ry] == [id(m) for seq in mod.mods for m in seq]

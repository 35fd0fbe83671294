"""Pin the complex128 oracle against the reference's own outputs (golden
vectors made by running qandle in tests/golden/make_golden.py), and against
finite differences / the parameter-shift rule for gradients.  CPU only."""
import json

import numpy as np
import pytest

from oracle import oracle
from qandle_gb300 import workloads
from tests import golden_io

# complex64 reference vs complex128 oracle: the reference's error per gate is
# about 1e-7; whole circuits stay well inside 1e-5 (the parity bar).
TOL = 2e-6


def test_gates_golden():
    z = golden_io.load("gates")
    for i in range(int(z["count"])):
        d = json.loads(str(z[f"g{i}_desc"]))
        gate = golden_io.parse_gate(d["gate"])
        inp = z[f"g{i}_in"]
        desc = {"n": d["n"], "batch": inp.shape[0] if inp.ndim == 2 else None,
                "gates": [gate], "inputs": {}}
        out = oracle.run(desc, state=inp, batch=inp.shape[0] if inp.ndim == 2 else 1)
        ref = z[f"g{i}_out"].reshape(out.shape)
        if gate[0] in ("cnot", "cz", "swap"):
            # permutations and sign flips move amplitudes exactly
            assert np.array_equal(out.astype(np.complex64), ref), (i, gate)
        else:
            assert np.abs(out - ref).max() < TOL, (i, gate)


def test_embeddings_golden():
    z = golden_io.load("embeddings")
    for i in range(int(z["count"])):
        d = json.loads(str(z[f"e{i}_desc"]))
        x = z[f"e{i}_x"]
        B = x.shape[0] if x.ndim == 2 else 1
        desc = {"n": d["n"], "batch": B, "gates": [("emb", d["rot"], "e", d["qubits"])],
                "inputs": {"e": x.reshape(B, -1)}}
        out = oracle.run(desc)
        ref = z[f"e{i}_out"].reshape(out.shape)
        assert np.abs(out - ref).max() < TOL, i


def test_measurements_golden():
    z = golden_io.load("measurements")
    for i in range(int(z["count"])):
        inp = z[f"m{i}_in"]
        st = inp.reshape(-1, inp.shape[-1]).astype(np.complex128)
        p0 = oracle.measure_p0(st)
        ref = z[f"m{i}_p0"]
        # measurements.py:123 squeezes: compare values, shapes are the
        # front end's business
        assert np.abs(p0.reshape(-1) - ref.reshape(-1)).max() < TOL
        assert np.abs((np.abs(st) ** 2).reshape(-1) - z[f"m{i}_joint"].reshape(-1)).max() < TOL


def test_sel_golden():
    z = golden_io.load("sel")
    for i in range(int(z["count"])):
        d = json.loads(str(z[f"s{i}_desc"]))
        n, depth, w = d["n"], d["depth"], z[f"s{i}_w"]
        gates = []
        for layer in range(depth):
            for q in range(n):
                for r, ax in enumerate(("rz", "ry", "rz")):
                    gates.append((ax, q, float(w[layer, q, r]), None))
            rng = layer % (n - 1) + 1
            for q in range(n):
                gates.append(("cnot", q, (q + rng) % n))
        inp = z[f"s{i}_in"]
        B = inp.shape[0] if inp.ndim == 2 else 1
        out = oracle.run({"n": n, "batch": B, "gates": gates, "inputs": {}}, state=inp, batch=B)
        assert np.abs(out - z[f"s{i}_out"].reshape(out.shape)).max() < 1e-5


def test_reupload_golden():
    z = golden_io.load("reupload")
    g = [("rx", 1, None, "r")]
    v, vb = float(z["v"]), z["vb"]
    out = oracle.run({"n": 3, "batch": 1, "gates": g, "inputs": {"r": np.float32(v)}},
                     state=z["inp_u"], batch=1)
    assert np.abs(out[0] - z["unb"]).max() < TOL
    out = oracle.run({"n": 3, "batch": 7, "gates": g, "inputs": {"r": vb}}, state=z["inp_b"])
    assert np.abs(out - z["bat_vec"]).max() < TOL
    out = oracle.run({"n": 3, "batch": 7, "gates": g, "inputs": {"r": np.float32(v)}},
                     state=z["inp_b"])
    assert np.abs(out - z["bat_scalar"]).max() < TOL
    # unbatched state with a batched input broadcasts (operators.py:293-297)
    out = oracle.run({"n": 3, "batch": 7, "gates": g, "inputs": {"r": vb}}, state=z["inp_u"])
    assert np.abs(out - z["unb_vec"]).max() < TOL


@pytest.mark.parametrize("name", ["plain_small", "sel_small", "brick_small", "deep_small"])
def test_circuits_golden(name):
    z = golden_io.load("circuits")
    desc = golden_io.circuit_desc(z, name)
    out = oracle.forward(desc)
    ref = z[f"{name}_out"]
    if desc["measure"] == "z":  # the golden file holds P0 for these
        out = oracle.measure_p0(oracle.run(desc))
    if out.shape != ref.shape and out.shape[1:] == ref.shape:
        # no per-sample input: the reference ran its unbatched |0..0> state
        ref = np.broadcast_to(ref, out.shape)
    assert np.abs(out.reshape(ref.shape) - ref).max() < 1e-5


def test_adjoint_vs_reference_autograd():
    z = golden_io.load("circuits")
    desc = golden_io.circuit_desc(z, "brick_small")
    st = oracle.run(desc)
    p0 = oracle.measure_p0(st)
    zexp = 2.0 * p0 - 1.0
    loss, dp0 = oracle.mse_z_grad(zexp, desc["targets"])
    assert abs(loss - float(z["brick_small_loss"])) < 1e-5
    dth, _, _ = oracle.adjoint(desc, dp0, "p0")
    assert np.abs(dth - z["brick_small_dtheta"]).max() < 1e-5

    desc = golden_io.circuit_desc(z, "sel_small")
    w = z["sel_small_weights"]
    dth, dnamed, _ = oracle.adjoint(desc, w, "p0")
    assert np.abs(dth - z["sel_small_dtheta"]).max() < 1e-5
    dx = dnamed["x"].copy()
    for q in range(desc["n"]):
        dx[:, q] += dnamed[f"up{q}"]
    assert np.abs(dx - z["sel_small_dx"]).max() < 1e-5


def test_adjoint_vs_finite_differences_and_shift():
    desc = workloads.adjoint_brick(n=5, batch=3, layers=3)
    t = desc["targets"]

    def loss_of(d):
        z_ = 2.0 * oracle.measure_p0(oracle.run(d)) - 1.0
        return float(((z_ - t) ** 2).mean())

    z0 = 2.0 * oracle.measure_p0(oracle.run(desc)) - 1.0
    _, dp0 = oracle.mse_z_grad(z0, t)
    dth, _, _ = oracle.adjoint(desc, dp0, "p0")
    slots = [i for i, g in enumerate(desc["gates"]) if g[0] in ("rx", "ry", "rz")]
    h = 1e-3
    for k in (0, 3, 7, len(slots) - 1):
        gi = slots[k]

        def with_theta(v):
            d = dict(desc)
            gs = list(d["gates"])
            g = gs[gi]
            gs[gi] = (g[0], g[1], v, None)
            d["gates"] = gs
            return d

        th = desc["gates"][gi][2]
        # angles are float32 in every executor: difference over the
        # representable step actually taken
        tp, tm = float(np.float32(th + h)), float(np.float32(th - h))
        fd = (loss_of(with_theta(tp)) - loss_of(with_theta(tm))) / (tp - tm)
        assert abs(fd - dth[k]) < 1e-6, (k, fd, dth[k])
        # parameter shift of the measured expectation (t = theta/2, shift pi/2)
        zp = 2.0 * oracle.measure_p0(oracle.run(with_theta(th + np.pi / 2))) - 1.0
        zm = 2.0 * oracle.measure_p0(oracle.run(with_theta(th - np.pi / 2))) - 1.0
        dz = (zp - zm) / 2.0
        # chain rule through the MSE with the unshifted residual
        ps = float((2.0 * (z0 - t) / z0.size * dz).sum())
        assert abs(ps - dth[k]) < 1e-7, (k, ps, dth[k])  # shifted angles round to float32


def test_oracle_special_gates_vs_reference():
    """Reset, Invert of every gate kind and Controlled rotations / U (fixed
    and per-sample angles) against the reference's outputs."""
    z = golden_io.load("special")
    for i in range(int(z["count"])):
        spec = json.loads(str(z[f"s{i}_spec"]))
        inp = z[f"s{i}_in"]
        ref = z[f"s{i}_out"]
        batch = inp.shape[0] if inp.ndim == 2 else 1
        inputs = {k[len(f"s{i}_kw_"):]: z[k] for k in z.files if k.startswith(f"s{i}_kw_")}
        desc = {"n": spec["n"], "batch": batch, "gates": golden_io.special_gates(spec), "inputs": inputs,
                "measure": "state"}
        st = oracle.run(desc, state=inp.reshape(batch, -1))
        got = st
        if spec.get("measure") == "probs":
            got = np.abs(st) ** 2
        assert np.abs(got.reshape(ref.shape) - ref).max() < 2e-5, (i, spec)


def test_oracle_controlled_gradients_vs_reference_autograd():
    z = golden_io.load("special")
    th = [float(v) for v in z["grad_thetas"]]
    desc = {"n": 4, "batch": 3, "inputs": {}, "measure": "p0",
            "gates": [("ry", 0, th[0], None), ("cnot", 0, 1), ("crx", 1, 2, th[1], None),
                      ("cry", 2, 3, th[2], None), ("crz", 3, 0, th[3], None)]}
    p0 = oracle.forward(desc, state=z["grad_in"])
    assert np.abs(p0 - z["grad_p0"]).max() < 1e-5
    w = np.broadcast_to(np.arange(1, 5, dtype=np.float64), (3, 4)).copy()
    dth, _, _ = oracle.adjoint(desc, w, "p0", state=z["grad_in"])
    assert np.abs(dth - z["grad_out"]).max() < 1e-4


def test_amplitude_formula_vs_reference():
    """The torch restatement used by the amplitude embedding's backward
    equals the reference's forward on every golden case (host-side logic)."""
    import torch

    from qandle_gb300 import plain

    z = golden_io.load("amplitude")
    for i in range(int(z["count"])):
        spec = json.loads(str(z[f"a{i}_spec"]))
        y = plain._amp_embed_torch(torch.tensor(z[f"a{i}_x"]), spec["n"], spec["pad"], spec["normalize"])
        assert np.abs(y.numpy() - z[f"a{i}_out"]).max() < 1e-6, spec


def test_amplitude_crop_vs_reference():
    """More features than amplitudes with a pad value: the reference cuts
    the features past 2^n (torch's pad with a negative width) before
    normalising.  The torch restatement equals the reference, and the
    feature count the kernel is given is 2^n; without a pad value other
    counts than 2^n are refused."""
    import torch

    from qandle_gb300 import plain

    z = golden_io.load("amplitude_crop")
    for i in range(int(z["count"])):
        spec = json.loads(str(z[f"c{i}_spec"]))
        x = torch.tensor(z[f"c{i}_x"])
        y = plain._amp_embed_torch(x, spec["n"], spec["pad"], spec["normalize"])
        assert np.abs(y.numpy() - z[f"c{i}_out"]).max() < 1e-6, spec
        assert plain.amp_embed_length(x.shape[-1], spec["n"], spec["pad"]) == 1 << spec["n"]
    assert plain.amp_embed_length(3, 3, 0.0) == 3
    assert plain.amp_embed_length(8, 3, None) == 8
    for length in (3, 9):
        with pytest.raises(ValueError):
            plain.amp_embed_length(length, 3, None)


def test_random_circuits_golden():
    """30 random circuits over every gate kind of the path (fixed and named
    rotations, U, CNOT, CZ, SWAP; 3..8 qubits, batch 3, seeded input states):
    the oracle equals the reference's output states."""
    from tests.golden import make_golden as mg

    z = golden_io.load("random_circuits")
    for name, (desc, psi) in mg.random_circuit_descs().items():
        out = oracle.run(desc, state=psi, batch=desc["batch"])
        assert np.abs(out - z[f"{name}_out"]).max() < TOL, name


def test_random_circuit_gradients_vs_reference_autograd():
    """The oracle's adjoint gradients (unnamed angles, named inputs) equal
    torch autograd through the reference for 12 random circuits over every
    gate kind, loss sum(W * joint probabilities)."""
    from tests.golden import make_golden as mg

    z = golden_io.load("random_grads")
    checked = 0
    for name, (desc, psi) in mg.random_circuit_descs().items():
        if f"{name}_w" not in z.files:
            continue
        d = dict(desc, measure="probs")
        dth, dnamed, _ = oracle.adjoint(d, z[f"{name}_w"].astype(np.float64), "probs", state=psi,
                                        batch=d["batch"])
        assert np.abs(dth - z[f"{name}_dtheta"]).max() < 1e-5, name
        for k in d["inputs"]:
            assert np.abs(dnamed[k] - z[f"{name}_dnamed_{k}"]).max() < 1e-5, (name, k)
        checked += 1
    assert checked == 12

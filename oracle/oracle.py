"""ctypes front of the complex128 CPU oracle (oracle/sv_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA engine.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU baseline leg use this module; the
product package never imports it.

It consumes the plain circuit descriptions of qandle_gb300/workloads.py and
restates the reference's semantics in complex128 (see the header of
sv_oracle.c for the reference file:line each rule follows).  Angles are
widened from float32 to float64 before t = theta / 2 is formed, so the oracle
is the exact-arithmetic answer for the float32 inputs the engine receives.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "libsv_oracle.so")
_SRC = os.path.join(_HERE, "sv_oracle.c")
_lock = threading.Lock()
_lib = None

KIND = {"rx": 0, "ry": 1, "rz": 2, "u": 3, "cnot": 4, "cz": 5, "swap": 6, "emb": 7, "crot": 8, "cu": 9,
        "reset": 10}
ROT = {"rx": 0, "ry": 1, "rz": 2, "x": 0, "y": 1, "z": 2}
SEED = {"p0": 0, "z": 0, "probs": 1, "state": 2}


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (OpenMP) into oracle/_build/."""
    os.makedirs(_BUILD, exist_ok=True)
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(_SRC):
        tmp = _SO + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-shared", "-fPIC", "-std=c11",
                               _SRC, "-o", tmp, "-lm"])
        os.replace(tmp, _SO)
    return _SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            _lib = ctypes.CDLL(build())
            P = ctypes.c_void_p
            I64, I = ctypes.c_int64, ctypes.c_int
            _lib.or_run.argtypes = [P, I64, I, P, I, P, P, I, P, P, I]
            _lib.or_measure_p0.argtypes = [P, I64, I, P]
            _lib.or_probs.argtypes = [P, I64, P]
            _lib.or_adjoint.argtypes = [P, I64, I, P, I, P, I, P, I, P, P, I, P, P, P, P, I]
        return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Lowered:
    """A description flattened to the oracle's record arrays."""

    def __init__(self, desc: dict, batch: int | None = None):
        self.n = desc["n"]
        self.batch = batch if batch is not None else (desc["batch"] or 1)
        recs, theta, umats, qlist = [], [], [], []
        named_cols = []  # list of per-sample float arrays [B]
        self.theta_gate = []  # gate index of each theta slot
        self.named_slots = []  # (name, column-in-input or None, col)
        inputs = desc.get("inputs", {})
        B = self.batch

        def add_named(name, j=None):
            v = np.asarray(inputs[name], dtype=np.float32)
            if j is not None:
                v = v[..., j]
            v = np.broadcast_to(v.astype(np.float64), (B,)) if v.ndim == 0 else v.astype(np.float64)
            if v.shape[0] != B:
                v = np.broadcast_to(v[:B], (B,))
            named_cols.append(np.ascontiguousarray(v))
            self.named_slots.append((name, j))
            return len(named_cols) - 1

        for gi, g in enumerate(desc["gates"]):
            k = g[0]
            if k in ("rx", "ry", "rz"):
                if g[3] is None:
                    recs.append([KIND[k], g[1], 0, 0, len(theta), 0])
                    theta.append(float(np.float32(g[2])))
                    self.theta_gate.append(gi)
                else:
                    col = add_named(g[3])
                    recs.append([KIND[k], g[1], 0, 1, col, 0])
            elif k == "u":
                m = np.asarray(g[2], dtype=np.complex64).astype(np.complex128).reshape(2, 2)
                recs.append([KIND[k], g[1], 0, 0, len(umats), 0])
                umats.append(np.stack([m.real, m.imag], -1).reshape(-1))
            elif k in ("cnot", "cz", "swap"):
                recs.append([KIND[k], g[1], g[2], 0, 0, 0])
            elif k in ("crx", "cry", "crz"):
                # controlled rotation: (kind, control, target, angle, name)
                axis = ROT[k[1:]]
                if g[4] is None:
                    recs.append([KIND["crot"], g[1], g[2], 0, len(theta), axis])
                    theta.append(float(np.float32(g[3])))
                    self.theta_gate.append(gi)
                else:
                    col = add_named(g[4])
                    recs.append([KIND["crot"], g[1], g[2], 1, col, axis])
            elif k == "cu":
                m = np.asarray(g[3], dtype=np.complex64).astype(np.complex128).reshape(2, 2)
                recs.append([KIND[k], g[1], g[2], 0, len(umats), 0])
                umats.append(np.stack([m.real, m.imag], -1).reshape(-1))
            elif k == "reset":
                recs.append([KIND[k], g[1], 0, 0, 0, 0])
            elif k == "emb":
                qs = list(g[3])
                first = None
                for j in range(len(qs)):
                    c = add_named(g[2], j)
                    first = c if first is None else first
                recs.append([KIND[k], ROT[g[1]], len(qs), 1, first if first is not None else 0,
                             len(qlist)])
                qlist.extend(qs)
            else:
                raise ValueError(f"unknown gate {k}")
        self.gates = np.ascontiguousarray(np.array(recs, dtype=np.int32).reshape(-1, 6))
        self.theta = np.ascontiguousarray(np.array(theta + [0.0], dtype=np.float64))
        self.ntheta = len(theta)
        self.umats = np.ascontiguousarray(
            np.concatenate(umats) if umats else np.zeros(8), dtype=np.float64)
        self.qlist = np.ascontiguousarray(np.array(qlist + [0], dtype=np.int32))
        self.ncols = len(named_cols)
        self.named = (np.ascontiguousarray(np.stack(named_cols, 1)) if named_cols
                      else np.zeros((B, 1)))


def run(desc: dict, state: np.ndarray | None = None, batch: int | None = None,
        nthreads: int = 0, lowered: Lowered | None = None) -> np.ndarray:
    """Final state, complex128 [B, 2^n]."""
    lo = lowered or Lowered(desc, batch)
    B, n = lo.batch, lo.n
    st = np.zeros((B, 1 << n, 2), dtype=np.float64)
    if state is None:
        st[:, 0, 0] = 1.0
    else:
        s = np.broadcast_to(np.asarray(state, dtype=np.complex128).reshape(-1, 1 << n), (B, 1 << n))
        st[..., 0] = s.real
        st[..., 1] = s.imag
    lib().or_run(_ptr(st), B, n, _ptr(lo.gates), lo.gates.shape[0], _ptr(lo.theta),
                 _ptr(lo.named), lo.ncols, _ptr(lo.umats), _ptr(lo.qlist), nthreads)
    return st[..., 0] + 1j * st[..., 1]


def measure_p0(state: np.ndarray) -> np.ndarray:
    st = np.ascontiguousarray(np.stack([state.real, state.imag], -1), dtype=np.float64)
    B, dim = state.shape
    n = dim.bit_length() - 1
    out = np.zeros((B, n), dtype=np.float64)
    lib().or_measure_p0(_ptr(st), B, n, _ptr(out))
    return out


def measure(desc: dict, state: np.ndarray) -> np.ndarray:
    m = desc.get("measure")
    if m == "probs":
        return np.abs(state) ** 2
    if m == "p0":
        return measure_p0(state)
    if m == "z":
        return 2.0 * measure_p0(state) - (np.abs(state) ** 2).sum(-1, keepdims=True)
    return state


def forward(desc: dict, state=None, batch=None, nthreads: int = 0) -> np.ndarray:
    return measure(desc, run(desc, state, batch, nthreads))


def adjoint(desc: dict, gout: np.ndarray, seed: str, state=None, batch=None,
            nthreads: int = 0):
    """Gradients by the adjoint method in complex128.

    Returns (dtheta [ntheta] summed over samples, dnamed dict name -> array
    shaped like the input, dstate [B, 2^n] complex in torch's convention)."""
    lo = Lowered(desc, batch)
    B, n = lo.batch, lo.n
    psi0 = None
    if state is not None:
        s = np.broadcast_to(np.asarray(state, dtype=np.complex128).reshape(-1, 1 << n), (B, 1 << n))
        psi0 = np.ascontiguousarray(np.stack([s.real, s.imag], -1))
    if seed == "state":
        g = np.asarray(gout, dtype=np.complex128).reshape(B, 1 << n)
        gbuf = np.ascontiguousarray(np.stack([g.real, g.imag], -1))
    else:
        gbuf = np.ascontiguousarray(np.asarray(gout, dtype=np.float64))
    dth = np.zeros(max(lo.ntheta, 1))
    dnm = np.zeros((B, max(lo.ncols, 1)))
    dps = np.zeros((B, 1 << n, 2))
    lib().or_adjoint(_ptr(psi0), B, n, _ptr(lo.gates), lo.gates.shape[0], _ptr(lo.theta),
                     lo.ntheta, _ptr(lo.named), lo.ncols, _ptr(lo.umats), _ptr(lo.qlist),
                     SEED[seed], _ptr(gbuf), _ptr(dth), _ptr(dnm), _ptr(dps), nthreads)
    dnamed = {}
    for col, (name, j) in enumerate(lo.named_slots):
        shape = np.asarray(desc["inputs"][name]).shape
        arr = dnamed.setdefault(name, np.zeros((B,) + tuple(shape[1:]) if len(shape) else (B,)))
        if j is None:
            arr += dnm[:, col] if arr.ndim == 1 else dnm[:, col][:, None]
        else:
            arr[:, j] += dnm[:, col]
    return dth[:lo.ntheta], dnamed, dps[..., 0] + 1j * dps[..., 1]


def mse_z_grad(z: np.ndarray, targets: np.ndarray) -> tuple[float, np.ndarray]:
    """Loss = mean((z - t)^2) with z = 2 P0 - 1; returns (loss, dL/dP0)."""
    d = z - targets
    loss = float((d ** 2).mean())
    dz = 2.0 * d / d.size
    return loss, 2.0 * dz

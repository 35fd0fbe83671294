"""Plain form: torch autograd Functions over the per-gate CUDA kernels.

Each Function clones its input (the reference's layers are out-of-place,
``state @ M``) and runs one in-place kernel pass on the clone.  Backward runs
the adjoint of the same kernel on the incoming gradient, plus a reduction
kernel for the angle gradient.  torch's complex gradient convention is used
throughout: grad = 2 dL/dz*.

States are viewed as [B, 2^n]; an unbatched [2^n] state is B = 1.
"""
from __future__ import annotations

import torch
from torch.autograd.function import once_differentiable

from . import _lib

AXES = {"x": 0, "y": 1, "z": 2, "rx": 0, "ry": 1, "rz": 2}


def _as_batched(state: torch.Tensor, n: int) -> torch.Tensor:
    _lib.require_cuda_state(state)
    if state.shape[-1] != (1 << n):
        raise ValueError(f"state has {state.shape[-1]} amplitudes, expected 2^{n}")
    return state.reshape(-1, 1 << n).contiguous()


def _scratch(nbytes: int, device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 16), dtype=torch.uint8, device=device)


class Rotation(torch.autograd.Function):
    """RX/RY/RZ by ``angle`` (float32; one value, or one per sample)."""

    @staticmethod
    def forward(ctx, state, angle, n, qubit, axis):
        st = _as_batched(state, n)
        B = st.shape[0]
        a = angle.to(device=st.device, dtype=torch.float32).reshape(-1).contiguous()
        per_sample = a.numel() > 1
        if per_sample and B == 1:
            st = st.expand(a.numel(), -1)
            B = a.numel()
        if per_sample and a.numel() != B:
            raise ValueError(f"named input has {a.numel()} values for a batch of {B}")
        out = st.clone()
        _lib.call("qg_apply_rotation", out.data_ptr(), B, n, qubit, axis, a.data_ptr(),
                  1 if per_sample else 0, 0, _lib.stream())
        ctx.save_for_backward(out, a)
        ctx.meta = (n, qubit, axis, per_sample, angle.shape, state.shape, B)
        if state.dim() == 1 and not per_sample:
            return out.reshape(state.shape)
        return out

    @staticmethod
    @once_differentiable
    def backward(ctx, g):
        out, a = ctx.saved_tensors
        n, qubit, axis, per_sample, ashape, sshape, B = ctx.meta
        g = g.reshape(B, 1 << n).contiguous()
        gin = dth = None
        if ctx.needs_input_grad[0]:
            gin = g.clone()
            _lib.call("qg_apply_rotation", gin.data_ptr(), B, n, qubit, axis, a.data_ptr(),
                      1 if per_sample else 0, 1, _lib.stream())
            orig_b = 1 if len(sshape) == 1 else sshape[0]
            if orig_b != B:  # the state was broadcast over per-sample angles
                gin = gin.sum(0, keepdim=True)
            gin = gin.reshape(sshape)
        if ctx.needs_input_grad[1]:
            scr = _scratch(_lib.load().qg_rotation_grad_scratch_bytes(B, n), g.device)
            dth = torch.empty(B if per_sample else 1, dtype=torch.float32, device=g.device)
            _lib.call("qg_rotation_grad", out.data_ptr(), g.data_ptr(), dth.data_ptr(), B, n, qubit,
                      axis, 1 if per_sample else 0, scr.data_ptr(), scr.numel(), _lib.stream())
            dth = dth.reshape(ashape)
        return gin, dth, None, None, None


class Matrix(torch.autograd.Function):
    """Fixed 2x2 ``row_matrix`` applied as state @ kron(.., M, ..)."""

    @staticmethod
    def forward(ctx, state, row_matrix, n, qubit):
        st = _as_batched(state, n)
        m = row_matrix.to(device=st.device, dtype=torch.complex64).contiguous()
        out = st.clone()
        _lib.call("qg_apply_matrix", out.data_ptr(), st.shape[0], n, qubit, m.data_ptr(), 0,
                  _lib.stream())
        ctx.save_for_backward(m)
        ctx.meta = (n, qubit, state.shape)
        return out.reshape(state.shape)

    @staticmethod
    @once_differentiable
    def backward(ctx, g):
        (m,) = ctx.saved_tensors
        n, qubit, sshape = ctx.meta
        gin = g.reshape(-1, 1 << n).contiguous().clone()
        _lib.call("qg_apply_matrix", gin.data_ptr(), gin.shape[0], n, qubit, m.data_ptr(), 1,
                  _lib.stream())
        return gin.reshape(sshape), None, None, None


class ControlledRotation(torch.autograd.Function):
    """Rotation on ``qubit`` where ``control`` is 1 (BuiltControlled with a
    rotation target, qandle/operators.py:486-503)."""

    @staticmethod
    def forward(ctx, state, angle, n, control, qubit, axis):
        st = _as_batched(state, n)
        B = st.shape[0]
        a = angle.to(device=st.device, dtype=torch.float32).reshape(-1).contiguous()
        per_sample = a.numel() > 1
        if per_sample and B == 1:
            st = st.expand(a.numel(), -1)
            B = a.numel()
        if per_sample and a.numel() != B:
            raise ValueError(f"named input has {a.numel()} values for a batch of {B}")
        out = st.clone()
        _lib.call("qg_apply_controlled_rotation", out.data_ptr(), B, n, control, qubit, axis, a.data_ptr(),
                  1 if per_sample else 0, 0, _lib.stream())
        ctx.save_for_backward(out, a)
        ctx.meta = (n, control, qubit, axis, per_sample, angle.shape, state.shape, B)
        if state.dim() == 1 and not per_sample:
            return out.reshape(state.shape)
        return out

    @staticmethod
    @once_differentiable
    def backward(ctx, g):
        out, a = ctx.saved_tensors
        n, control, qubit, axis, per_sample, ashape, sshape, B = ctx.meta
        g = g.reshape(B, 1 << n).contiguous()
        gin = dth = None
        if ctx.needs_input_grad[0]:
            gin = g.clone()
            _lib.call("qg_apply_controlled_rotation", gin.data_ptr(), B, n, control, qubit, axis, a.data_ptr(),
                      1 if per_sample else 0, 1, _lib.stream())
            orig_b = 1 if len(sshape) == 1 else sshape[0]
            if orig_b != B:
                gin = gin.sum(0, keepdim=True)
            gin = gin.reshape(sshape)
        if ctx.needs_input_grad[1]:
            scr = _scratch(_lib.load().qg_rotation_grad_scratch_bytes(B, n), g.device)
            dth = torch.empty(B if per_sample else 1, dtype=torch.float32, device=g.device)
            _lib.call("qg_controlled_rotation_grad", out.data_ptr(), g.data_ptr(), dth.data_ptr(), B, n, control,
                      qubit, axis, 1 if per_sample else 0, scr.data_ptr(), scr.numel(), _lib.stream())
            dth = dth.reshape(ashape)
        return gin, dth, None, None, None, None


class ControlledMatrix(torch.autograd.Function):
    """Fixed 2x2 on ``qubit`` where ``control`` is 1."""

    @staticmethod
    def forward(ctx, state, row_matrix, n, control, qubit):
        st = _as_batched(state, n)
        m = row_matrix.to(device=st.device, dtype=torch.complex64).contiguous()
        out = st.clone()
        _lib.call("qg_apply_controlled_matrix", out.data_ptr(), st.shape[0], n, control, qubit, m.data_ptr(), 0,
                  _lib.stream())
        ctx.save_for_backward(m)
        ctx.meta = (n, control, qubit, state.shape)
        return out.reshape(state.shape)

    @staticmethod
    @once_differentiable
    def backward(ctx, g):
        (m,) = ctx.saved_tensors
        n, control, qubit, sshape = ctx.meta
        gin = g.reshape(-1, 1 << n).contiguous().clone()
        _lib.call("qg_apply_controlled_matrix", gin.data_ptr(), gin.shape[0], n, control, qubit, m.data_ptr(), 1,
                  _lib.stream())
        return gin.reshape(sshape), None, None, None, None


def _reset_torch(x: torch.Tensor, n: int, qubit: int) -> torch.Tensor:
    """The reset of qandle/operators.py:612-623 as torch ops on [B, 2^n]
    (used for its backward: the same formula, differentiated by torch)."""
    v = x.reshape(x.shape[0], 1 << qubit, 2, 1 << (n - 1 - qubit))
    a0, a1 = v[:, :, 0, :], v[:, :, 1, :]
    nrm = torch.sqrt(a0.abs() ** 2 + a1.abs() ** 2)
    scale = nrm / (a0.abs() + 1e-7)
    return torch.stack([a0 * scale, torch.zeros_like(a1)], 2).reshape(x.shape)


class Reset(torch.autograd.Function):
    """Reset of ``qubit`` keeping the norm (qandle/operators.py:603-651):
    forward on the CUDA kernel, backward through the same formula."""

    @staticmethod
    def forward(ctx, state, n, qubit):
        st = _as_batched(state, n)
        out = st.clone()
        _lib.call("qg_reset", out.data_ptr(), st.shape[0], n, qubit, _lib.stream())
        ctx.save_for_backward(st)
        ctx.meta = (n, qubit, state.shape)
        return out.reshape(state.shape)

    @staticmethod
    @once_differentiable
    def backward(ctx, g):
        (st,) = ctx.saved_tensors
        n, qubit, sshape = ctx.meta
        with torch.enable_grad():
            x = st.detach().requires_grad_(True)
            y = _reset_torch(x, n, qubit)
            (gin,) = torch.autograd.grad(y, x, g.reshape(y.shape))
        return gin.reshape(sshape), None, None


def _amp_embed_torch(x: torch.Tensor, n: int, pad_with, normalize: bool) -> torch.Tensor:
    """AmplitudeEmbeddingBuilt.forward (qandle/embeddings.py:50-62) as torch
    ops, for the backward of AmpEmbed."""
    pad_len = (1 << n) - x.shape[-1]
    if pad_len:
        x = torch.nn.functional.pad(x, (0, pad_len), mode="constant", value=pad_with)
    if normalize:
        x = torch.nn.functional.normalize(x, p=2, dim=-1)
    return torch.complex(x, torch.zeros_like(x))


def amp_embed_length(num_features: int, n: int, pad_with) -> int:
    """How many features of each row the amplitude embedding reads.  With a
    pad value the reference pads to 2^n with torch's pad, whose negative
    width cuts the features past 2^n (qandle/embeddings.py:50-62); without
    one it passes the features through unchanged, which is a state only when
    there are exactly 2^n of them, so other counts are refused here."""
    dim = 1 << n
    if pad_with is None:
        if num_features != dim:
            raise ValueError(f"{num_features} features for {n} qubits need pad_with (or exactly {dim})")
        return dim
    return min(num_features, dim)


class AmpEmbed(torch.autograd.Function):
    """AmplitudeEmbedding: real features padded to 2^n and optionally
    normalised, as a complex64 state (CUDA kernel); the backward
    differentiates the same formula."""

    @staticmethod
    def forward(ctx, x, n, pad_with, normalize):
        xf = x.to(dtype=torch.float32)
        lead = xf.shape[:-1]
        x2 = xf.reshape(-1, xf.shape[-1]).contiguous()
        if not x2.is_cuda:
            raise RuntimeError("qandle_gb300 runs on CUDA tensors only; move the features with .to('cuda')")
        B, L = x2.shape
        used = amp_embed_length(L, n, pad_with)
        out = torch.empty(B, 1 << n, dtype=torch.complex64, device=x2.device)
        lib = _lib.load()
        scr = _scratch(lib.qg_amplitude_embedding_scratch_bytes(B, used) if normalize else 16, x2.device)
        # rows of x are L apart; the first `used` features of each are read
        _lib.call("qg_amplitude_embedding", out.data_ptr(), x2.data_ptr(), L, B, n, used,
                  float(pad_with or 0.0), 1 if normalize else 0, scr.data_ptr(), scr.numel(), _lib.stream())
        ctx.save_for_backward(x2)
        ctx.meta = (n, pad_with, normalize, x.shape, x.dtype)
        return out.reshape(*lead, 1 << n)

    @staticmethod
    @once_differentiable
    def backward(ctx, g):
        (x2,) = ctx.saved_tensors
        n, pad_with, normalize, xshape, xdtype = ctx.meta
        with torch.enable_grad():
            xx = x2.detach().requires_grad_(True)
            y = _amp_embed_torch(xx, n, pad_with, normalize)
            (gx,) = torch.autograd.grad(y, xx, g.reshape(y.shape))
        return gx.reshape(xshape).to(xdtype), None, None, None


_PERM = {"cnot": "qg_apply_cnot", "cz": "qg_apply_cz", "swap": "qg_apply_swap"}


class Permutation(torch.autograd.Function):
    """CNOT / CZ / SWAP: exact amplitude moves and sign flips (involutions,
    so the backward applies the same kernel)."""

    @staticmethod
    def forward(ctx, state, n, kind, qa, qb):
        st = _as_batched(state, n)
        out = st.clone()
        if not (kind == "swap" and qa == qb):
            _lib.call(_PERM[kind], out.data_ptr(), st.shape[0], n, qa, qb, _lib.stream())
        ctx.meta = (n, kind, qa, qb, state.shape)
        return out.reshape(state.shape)

    @staticmethod
    @once_differentiable
    def backward(ctx, g):
        n, kind, qa, qb, sshape = ctx.meta
        gin = g.reshape(-1, 1 << n).contiguous().clone()
        if not (kind == "swap" and qa == qb):
            _lib.call(_PERM[kind], gin.data_ptr(), gin.shape[0], n, qa, qb, _lib.stream())
        return gin.reshape(sshape), None, None, None, None


class AngleEmbed(torch.autograd.Function):
    """Product state prod_j R(x_j) on qubits[j] |0..0>; x: [B, k]."""

    @staticmethod
    def forward(ctx, x, n, qubits, axis):
        if not x.is_cuda:
            raise RuntimeError("qandle_gb300 runs on CUDA tensors only; the embedding input is on "
                               f"{x.device}")
        xb = x.to(torch.float32).reshape(-1, len(qubits)).contiguous()
        B = xb.shape[0]
        out = torch.empty(B, 1 << n, dtype=torch.complex64, device=x.device)
        scr = _scratch(_lib.load().qg_angle_embedding_scratch_bytes(B, n), x.device)
        qarr = (_lib.c_int * max(1, len(qubits)))(*qubits)
        _lib.call("qg_angle_embedding", out.data_ptr(), xb.data_ptr(), len(qubits), B, n, qarr,
                  len(qubits), axis, scr.data_ptr(), scr.numel(), _lib.stream())
        ctx.save_for_backward(out)
        ctx.meta = (n, tuple(qubits), axis, x.shape, B)
        return out

    @staticmethod
    @once_differentiable
    def backward(ctx, g):
        (out,) = ctx.saved_tensors
        n, qubits, axis, xshape, B = ctx.meta
        if not ctx.needs_input_grad[0]:
            return None, None, None, None
        g = g.reshape(B, 1 << n).contiguous()
        dx = torch.empty(B, len(qubits), dtype=torch.float32, device=g.device)
        scr = _scratch(_lib.load().qg_rotation_grad_scratch_bytes(B, n), g.device)
        col = torch.empty(B, dtype=torch.float32, device=g.device)
        for j, q in enumerate(qubits):
            _lib.call("qg_rotation_grad", out.data_ptr(), g.data_ptr(), col.data_ptr(), B, n, q,
                      axis, 1, scr.data_ptr(), scr.numel(), _lib.stream())
            dx[:, j] = col
        return dx.reshape(xshape), None, None, None


class MeasureP0(torch.autograd.Function):
    """P(qubit q = 0) -> [B, n] float32."""

    @staticmethod
    def forward(ctx, state, n):
        st = _as_batched(state, n)
        B = st.shape[0]
        out = torch.empty(B, n, dtype=torch.float32, device=st.device)
        scr = _scratch(_lib.load().qg_measure_p0_scratch_bytes(B, n), st.device)
        _lib.call("qg_measure_p0", st.data_ptr(), out.data_ptr(), B, n, scr.data_ptr(), scr.numel(),
                  _lib.stream())
        ctx.save_for_backward(st)
        ctx.meta = (n, state.shape)
        return out

    @staticmethod
    @once_differentiable
    def backward(ctx, g):
        (st,) = ctx.saved_tensors
        n, sshape = ctx.meta
        g = g.to(torch.float32).contiguous()
        gin = torch.empty_like(st)
        _lib.call("qg_measure_p0_backward", st.data_ptr(), g.data_ptr(), gin.data_ptr(),
                  st.shape[0], n, _lib.stream())
        return gin.reshape(sshape), None


class Probs(torch.autograd.Function):
    """|psi|^2, same shape as the state, float32."""

    @staticmethod
    def forward(ctx, state):
        _lib.require_cuda_state(state)
        st = state.contiguous()
        out = torch.empty(st.shape, dtype=torch.float32, device=st.device)
        _lib.call("qg_probs", st.data_ptr(), out.data_ptr(), st.numel(), _lib.stream())
        ctx.save_for_backward(st)
        return out

    @staticmethod
    @once_differentiable
    def backward(ctx, g):
        (st,) = ctx.saved_tensors
        g = g.to(torch.float32).contiguous()
        gin = torch.empty_like(st)
        _lib.call("qg_probs_backward", st.data_ptr(), g.data_ptr(), gin.data_ptr(), st.numel(),
                  _lib.stream())
        return gin


def _angle_buffer(angle, device):
    return torch.as_tensor(angle).to(device=device, dtype=torch.float32).reshape(-1).contiguous()


def apply_rotation_(st: torch.Tensor, n: int, qubit: int, axis: int, angle) -> torch.Tensor:
    """In-place rotation on a contiguous [B, 2^n] buffer (no autograd)."""
    a = _angle_buffer(angle, st.device)
    per = a.numel() > 1
    if per and st.shape[0] == 1 and a.numel() > 1:
        st = st.expand(a.numel(), -1).contiguous()
    _lib.call("qg_apply_rotation", st.data_ptr(), st.shape[0], n, qubit, axis, a.data_ptr(),
              1 if per else 0, 0, _lib.stream())
    return st


def run_layers_inplace(layers, state: torch.Tensor | None, n: int, kwargs: dict,
                       initial: torch.Tensor) -> torch.Tensor:
    """The plain form without autograd: one in-place kernel pass per gate on a
    single working buffer (the buffer is a copy; the caller's state is not
    modified).  Layers are the built modules of UnsplittedCircuit."""
    st = None
    src = initial if state is None else state
    unbatched = src.dim() == 1
    for mod in layers:
        name = type(mod).__name__
        if name in ("AngleEmbeddingBuilt", "AmplitudeEmbeddingBuilt"):
            st = mod(None, **kwargs)
            unbatched = st.dim() == 1
            st = st.reshape(-1, 1 << n)
            continue
        if st is None:
            _lib.require_cuda_state(src)
            st = src.reshape(-1, 1 << n).contiguous().clone()
        if name in ("BuiltRX", "BuiltRY", "BuiltRZ"):
            prev = st.shape[0]
            st = apply_rotation_(st, n, mod.qubit, mod.axis, mod.angle(**kwargs))
            if st.shape[0] != prev:
                unbatched = False
        elif name == "BuiltU":
            m = mod._m.to(st.device).contiguous()
            _lib.call("qg_apply_matrix", st.data_ptr(), st.shape[0], n, mod.qubit, m.data_ptr(), 0,
                      _lib.stream())
        elif name in ("BuiltCNOT", "BuiltCZ"):
            _lib.call(_PERM["cnot" if name == "BuiltCNOT" else "cz"], st.data_ptr(), st.shape[0], n,
                      mod.c, mod.t, _lib.stream())
        elif name == "BuiltSWAP":
            if mod.a != mod.b:
                _lib.call("qg_apply_swap", st.data_ptr(), st.shape[0], n, mod.a, mod.b, _lib.stream())
        elif name in ("BuiltInvert", "BuiltControlled", "BuiltReset"):
            prev = st.shape[0]
            st = (mod(st, **kwargs) if getattr(mod, "named", False) else mod(st)).reshape(-1, 1 << n)
            if st.shape[0] != prev:
                unbatched = False
        elif _composite(mod, n) is not None:
            st = run_layers_inplace(_composite(mod, n), st, n, kwargs, initial)
        else:
            # measurements: their own (out-of-place) forward ends the loop
            return mod(st.reshape(1 << n) if unbatched else st)
    if st is None:
        st = src.reshape(-1, 1 << n).clone()
    return st.reshape(1 << n) if unbatched else st


def _composite(mod, n: int):
    """The layers a composite layer runs, in order, or None for a single
    layer: a built ansatz's applied_gates (the reference's built SEL: its
    mods), a nested circuit's layers (on the same number of qubits)."""
    if hasattr(mod, "applied_gates"):
        return list(mod.applied_gates)
    if hasattr(mod, "mods"):
        return list(mod.mods)
    inner = getattr(mod, "circuit", None)
    if inner is not None and hasattr(inner, "layers") and hasattr(mod, "num_qubits"):
        if mod.num_qubits != n:
            raise ValueError(f"a nested circuit on {mod.num_qubits} qubits inside one on {n}")
        return list(inner.layers)
    return None


def _flat_layers(layers, n: int):
    out = []
    for mod in layers:
        sub = _composite(mod, n)
        if sub is not None:
            out.extend(_flat_layers(sub, n))
        else:
            out.append(mod)
    return out


def adjoint_per_gate(layers, n: int, grad_p0: torch.Tensor, state: torch.Tensor | None = None,
                     kwargs: dict | None = None, initial: torch.Tensor | None = None) -> list:
    """Adjoint gradient with one kernel pass per gate and state (the plain
    form of the adjoint): forward in place, then for every gate in reverse
    the angle gradient Im<lam|P|psi> (a reduction kernel) and the inverse
    gate on psi and on the cotangent.  The circuit must end with
    MeasureProbability; grad_p0 is dL/dP0 [B, n].  Returns dL/dangle for the
    unnamed rotations in layer order.  Shares no code with the fused engine
    and serves as its per-gate baseline."""
    kwargs = kwargs or {}
    flat = _flat_layers(layers, n)
    gates = [m for m in flat if type(m).__name__ not in ("MeasureProbabilityBuilt",)]
    with torch.no_grad():
        psi = run_layers_inplace(gates, state, n, kwargs, initial if initial is not None else state)
        psi = psi.reshape(-1, 1 << n).contiguous()
        B = psi.shape[0]
        g = torch.empty_like(psi)
        gp = grad_p0.to(torch.float32).reshape(B, n).contiguous()
        _lib.call("qg_measure_p0_backward", psi.data_ptr(), gp.data_ptr(), g.data_ptr(), B, n,
                  _lib.stream())
        scr = _scratch(_lib.load().qg_rotation_grad_scratch_bytes(B, n), psi.device)
        grads = {}
        one = torch.empty(1, dtype=torch.float32, device=psi.device)
        for mod in reversed(gates):
            name = type(mod).__name__
            if name in ("BuiltRX", "BuiltRY", "BuiltRZ"):
                a = _angle_buffer(mod.angle(**kwargs), psi.device)
                per = a.numel() > 1
                if not mod.named:
                    _lib.call("qg_rotation_grad", psi.data_ptr(), g.data_ptr(), one.data_ptr(), B, n,
                              mod.qubit, mod.axis, 0, scr.data_ptr(), scr.numel(), _lib.stream())
                    grads[id(mod)] = one.clone()
                for buf in (psi, g):
                    _lib.call("qg_apply_rotation", buf.data_ptr(), B, n, mod.qubit, mod.axis, a.data_ptr(),
                              1 if per else 0, 1, _lib.stream())
            elif name == "BuiltU":
                m = mod._m.to(psi.device).contiguous()
                for buf in (psi, g):
                    _lib.call("qg_apply_matrix", buf.data_ptr(), B, n, mod.qubit, m.data_ptr(), 1, _lib.stream())
            elif name in ("BuiltCNOT", "BuiltCZ"):
                for buf in (psi, g):
                    _lib.call(_PERM["cnot" if name == "BuiltCNOT" else "cz"], buf.data_ptr(), B, n, mod.c, mod.t,
                              _lib.stream())
            elif name == "BuiltSWAP":
                if mod.a != mod.b:
                    for buf in (psi, g):
                        _lib.call("qg_apply_swap", buf.data_ptr(), B, n, mod.a, mod.b, _lib.stream())
            elif name == "AngleEmbeddingBuilt":
                break
            else:
                raise ValueError(f"adjoint_per_gate cannot handle {name}")
        return [grads[id(m)] for m in gates if id(m) in grads]

"""CPU emulator of planned fused programs (test infrastructure).

Executes the op lists the planner emits (qg_program_pass / qg_program_slots)
on a complex128 state, tile by tile, in the tile's local-index view: an
OP_MAP exchange does not move data in that view, it only changes which local
bit each register position names.  This checks the planner's tile choice,
reordering, slot merging and op encoding on the CPU; the CUDA kernels'
mechanics (bulk copies, swizzled exchanges, thread mapping) are checked on
the GPU against the oracle.
"""
import numpy as np

OP_MAP, OP_MAT, OP_DIAG, OP_CX, OP_CZ, OP_SWAP, OP_GRAD, OP_XMAT = 1, 2, 3, 4, 5, 6, 7, 8
# OP_XMAT applies a register's pending X, a representation detail of the
# kernels: in the emulator's logical view it changes nothing
LOC_REG = 0x100
OPF_PER_SAMPLE, OPF_GRAD = 1, 2
INIT_LOAD, INIT_ZERO, INIT_EMBED = 0, 1, 2
EPI_STORE, EPI_PROBS, EPI_P0 = 1, 2, 4


def row_matrix(kind, theta):
    t = 0.5 * float(theta)
    c, s = np.cos(t), np.sin(t)
    if kind == 0:
        return np.array([[c, -1j * s], [-1j * s, c]])
    if kind == 1:
        return np.array([[c, s], [-s, c]], dtype=complex)
    return np.array([[c - 1j * s, 0], [0, c + 1j * s]])


def slot_tables(prog, backward, params, named, umats, B):
    """shared [S,2,2], per-sample [B,P,2,2] complex128 from the slot chains."""
    slots = prog.slots(backward)
    ns = sum(1 for s in slots if not s[0])
    nps = sum(1 for s in slots if s[0])
    shared = np.zeros((max(ns, 1), 2, 2), complex)
    ps = np.zeros((B, max(nps, 1), 2, 2), complex)
    for per_sample, ti, chain in slots:
        for b in range(B if per_sample else 1):
            m = np.eye(2, dtype=complex)
            for kind, src, idx, dag in chain:
                if kind == 3:
                    g = np.asarray(umats[idx], dtype=complex).reshape(2, 2)
                else:
                    th = params[idx] if src == 0 else named[b, idx]
                    g = row_matrix(kind, th)
                if dag:
                    g = g.conj().T
                m = m @ g
            if per_sample:
                ps[b, ti] = m
            else:
                shared[ti] = m
    return shared, ps


def tile_index(pd, n, B):
    """Global flat amplitude index of every (tile, local index); -1 = no sample."""
    TB, nq = pd["tile_bits"], pd["nq_tile"]
    j = np.arange(1 << TB)
    if n >= TB:
        off = np.zeros(1 << TB, dtype=np.int64)
        for k, g in enumerate(pd["gbit"]):
            off |= ((j >> k) & 1).astype(np.int64) << g
        tps = 1 << (n - TB)
        t = np.arange(tps)
        fv = np.zeros(tps, dtype=np.int64)
        for k, g in enumerate(pd["fixed_gbit"]):
            fv |= ((t >> k) & 1).astype(np.int64) << g
        base = (np.arange(B, dtype=np.int64)[:, None] << n) + fv[None, :]
        return base.reshape(-1, 1) + off[None, :]
    spt = 1 << (TB - n)
    ntiles = -(-B // spt)
    smp = np.arange(ntiles)[:, None] * spt + (j[None, :] >> n)
    idx = (smp << n) + (j[None, :] & ((1 << n) - 1))
    return np.where(smp < B, idx, -1)


def _bit(idx, lb_or_g, n, local, j):
    if local:
        return ((j >> lb_or_g) & 1).astype(bool)[None, :].repeat(idx.shape[0], 0)
    return (((np.where(idx < 0, 0, idx) & ((1 << n) - 1)) >> lb_or_g) & 1).astype(bool)


def _loc_bit(loc, regl, idx, n, j):
    if loc & LOC_REG:
        return _bit(idx, regl[loc & 7], n, True, j)
    return _bit(idx, loc, n, False, j)


def _decode(y):
    return [(y >> (4 * k)) & 15 for k in range(5)]


def _apply(T, op, regl, idx, n, j, samples, shared, ps, grads=None, lam=None):
    """Apply one op to tile array(s) T (and lam for the backward)."""
    code = op[0]
    arrs = [T] if lam is None else [T, lam]
    if code in (OP_MAT, OP_GRAD):
        lb = regl[op[1]]
        j0 = j[((j >> lb) & 1) == 0]
        j1 = j0 | (1 << lb)
        if code == OP_GRAD or (op[3] & OPF_GRAD):
            axis = op[2] if code == OP_GRAD else (op[3] >> 8) & 3
            slot = op[3] if code == OP_GRAD else op[3] >> 12
            p0, p1 = T[:, j0], T[:, j1]
            if axis == 0:
                q0, q1 = p1, p0
            elif axis == 1:
                q0, q1 = -1j * p1, 1j * p0
            else:
                q0, q1 = p0, -p1
            contrib = (np.conj(lam[:, j0]) * q0 + np.conj(lam[:, j1]) * q1).imag
            s = samples[:, j0]
            for (tile, k), v in np.ndenumerate(contrib):
                if s[tile, k] >= 0:
                    grads.setdefault(slot, np.zeros(ps.shape[0]))[s[tile, k]] += v
            if code == OP_GRAD:
                return
        if op[3] & OPF_PER_SAMPLE:
            m = ps[np.maximum(samples[:, j0], 0), op[2]]  # [tiles, len, 2, 2]
        else:
            m = np.broadcast_to(shared[op[2]], (T.shape[0], len(j0), 2, 2))
        for A in arrs:
            a0, a1 = A[:, j0].copy(), A[:, j1].copy()
            A[:, j0] = a0 * m[..., 0, 0] + a1 * m[..., 1, 0]
            A[:, j1] = a0 * m[..., 0, 1] + a1 * m[..., 1, 1]
    elif code == OP_DIAG:
        if op[3] & OPF_PER_SAMPLE:
            m = ps[np.maximum(samples, 0), op[2]]
        else:
            m = np.broadcast_to(shared[op[2]], T.shape + (2, 2))
        b = _loc_bit(op[1], regl, idx, n, j)
        for A in arrs:
            A *= np.where(b, m[..., 1, 1], m[..., 0, 0])
    elif code == OP_CX:
        lb = regl[op[1]]
        j0 = j[((j >> lb) & 1) == 0]
        j1 = j0 | (1 << lb)
        c = _loc_bit(op[2], regl, idx, n, j)[:, j0]
        for A in arrs:
            a0, a1 = A[:, j0].copy(), A[:, j1].copy()
            A[:, j0] = np.where(c, a1, a0)
            A[:, j1] = np.where(c, a0, a1)
    elif code == OP_CZ:
        c = _loc_bit(op[1], regl, idx, n, j) & _loc_bit(op[2], regl, idx, n, j)
        for A in arrs:
            A *= np.where(c, -1.0, 1.0)
    elif code == OP_SWAP:
        l0, l1 = regl[op[1]], regl[op[2]]
        js = j[(((j >> l0) & 1) == 1) & (((j >> l1) & 1) == 0)]
        jt = js ^ (1 << l0) ^ (1 << l1)
        for A in arrs:
            a, b = A[:, js].copy(), A[:, jt].copy()
            A[:, js], A[:, jt] = b, a


def run_forward(prog, n, B, params, named, umats, state=None, embed=None):
    """Final state [B, 2^n] and checkpoints of an emulated forward.
    embed: per-sample per-qubit factors [B, n, 2] (column vectors), or None."""
    shared, ps = slot_tables(prog, False, params, named, umats, B)
    st = np.zeros((B, 1 << n), complex)
    if state is not None:
        st[:] = state
    elif embed is None:
        st[:, 0] = 1.0
    ckpts = {}
    for p, pd in enumerate(prog.passes(False)):
        idx = tile_index(pd, n, B)
        j = np.arange(1 << pd["tile_bits"])
        valid = idx >= 0
        samples = np.where(valid, idx >> n, -1)
        if p == 0 and pd["init"] == INIT_EMBED:
            T = np.ones(idx.shape, complex)
            amp = np.where(valid, idx, 0) & ((1 << n) - 1)
            for q in range(n):
                bit = (amp >> (n - 1 - q)) & 1
                T *= embed[np.maximum(samples, 0), q, bit]
            regl = _decode(pd["init_map"][0])
        else:
            T = np.where(valid, st.reshape(-1)[np.maximum(idx, 0)], 0)
            regl = list(range(5, 5 + prog.reg_bits))
        for op in pd["ops"]:
            if op[0] == OP_MAP:
                regl = _decode(op[1])
            else:
                _apply(T, op, regl, idx, n, j, samples, shared, ps)
        if pd["epi"] & EPI_STORE or pd["ckpt"] >= 0 or True:
            flat = st.reshape(-1)
            flat[idx[valid]] = T[valid]
        if pd["ckpt"] >= 0:
            ckpts[pd["ckpt"]] = st.copy()
    return st, ckpts


def run_backward(prog, n, B, params, named, umats, psi, lam, ckpts, grad_targets):
    """Emulated adjoint sweep; returns (dparams, dnamed [B, ncols], lam_final)."""
    shared, ps = slot_tables(prog, True, params, named, umats, B)
    psi = psi.copy()
    lam = lam.copy()
    grads = {}
    for pd in prog.passes(True):
        src = ckpts[pd["psi_from_ckpt"]] if pd["psi_from_ckpt"] >= 0 else psi
        idx = tile_index(pd, n, B)
        j = np.arange(1 << pd["tile_bits"])
        valid = idx >= 0
        samples = np.where(valid, idx >> n, -1)
        T = np.where(valid, src.reshape(-1)[np.maximum(idx, 0)], 0)
        L = np.where(valid, lam.reshape(-1)[np.maximum(idx, 0)], 0)
        regl = list(range(5, 5 + 4))  # the backward keeps 16 amplitudes of psi and lambda per thread
        for op in pd["ops"]:
            if op[0] == OP_MAP:
                regl = _decode(op[1])
            else:
                _apply(T, op, regl, idx, n, j, samples, shared, ps, grads=grads, lam=L)
        psi.reshape(-1)[idx[valid]] = T[valid]
        lam.reshape(-1)[idx[valid]] = L[valid]
    nparams = max([t[1] + 1 for t in grad_targets if t[0] == 0] + [0])
    ncols = max([t[1] + 1 for t in grad_targets if t[0] == 1] + [0])
    dp = np.zeros(nparams)
    dn = np.zeros((B, ncols))
    for slot, v in grads.items():
        s, i = grad_targets[slot]
        if s == 0:
            dp[i] += v.sum()
        else:
            dn[:, i] += v
    return dp, dn, lam

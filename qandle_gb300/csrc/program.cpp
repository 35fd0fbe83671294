// Gate-fusion planner and program objects of the fused engine (host C++).
//
// A program is the lowered gate list of one circuit (the layers that
// UnsplittedCircuit.forward runs one by one, qandle/qcircuit.py:163-174)
// planned into passes.  Each pass loads a tile of 2^TB amplitudes spanning TB
// qubits (the low `low_bits` qubits, contiguous in memory, plus up to `k`
// strided ones), applies every gate that can act inside the tile, and writes
// the tile back: one HBM round trip for many gates.
//
// Inside a pass, gates act on amplitudes held in registers (32 per thread,
// spanning 5 "register" qubits); phases change which tile qubits are register
// qubits through a shared-memory exchange.  Gates may be reordered across a
// pass or phase boundary only where they commute: two gates commute when, on
// every qubit they share, both act diagonally in the Z basis (RZ, CZ, a CNOT
// control) or both in the X basis (RX, a CNOT target).  A gate's requirements:
// a non-diagonal single-qubit gate or a CNOT target needs its qubit inside the
// tile (and in registers); diagonal gates and CNOT controls may sit anywhere,
// since their effect only depends on the basis index.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "engine.h"
#include "jit.h"
#include "qandle_gb300.h"

namespace qg {

void set_error(const std::string& msg);

namespace {

enum GKind { K_ROT = 0, K_U = 1, K_CNOT = 2, K_CZ = 3, K_SWAP = 4, K_EMBED = 5 };

struct LGate {
    int kind = 0, axis = 0;
    int b0 = -1, b1 = -1;  // global bit positions
    int src = 0, idx = 0;  // angle / matrix source
    bool diag = false;
    bool grad = false;     // backward: accumulate a gradient for this gate
    int grad_slot = -1;
};

// per-bit action types for the commutation test
constexpr int T_Z = 1, T_X = 2, T_G = 4;

struct Touch {
    int bit[2];
    int type[2];
    int count;
};

Touch touches(const LGate& g) {
    Touch t{{-1, -1}, {0, 0}, 0};
    switch (g.kind) {
        case K_ROT:
            t.bit[0] = g.b0;
            t.type[0] = g.axis == 0 ? T_X : (g.axis == 2 ? T_Z : T_G);
            t.count = 1;
            break;
        case K_U:
            t.bit[0] = g.b0;
            t.type[0] = g.diag ? T_Z : T_G;
            t.count = 1;
            break;
        case K_CNOT:
            t.bit[0] = g.b0;
            t.type[0] = T_Z;
            t.bit[1] = g.b1;
            t.type[1] = T_X;
            t.count = 2;
            break;
        case K_CZ:
            t.bit[0] = g.b0;
            t.type[0] = T_Z;
            t.bit[1] = g.b1;
            t.type[1] = T_Z;
            t.count = 2;
            break;
        case K_SWAP:
            t.bit[0] = g.b0;
            t.type[0] = T_G;
            t.bit[1] = g.b1;
            t.type[1] = T_G;
            t.count = 2;
            break;
        case K_EMBED:  // backward gradient of one embedded angle: acts like its rotation
            t.bit[0] = g.b0;
            t.type[0] = g.axis == 0 ? T_X : (g.axis == 2 ? T_Z : T_G);
            t.count = 1;
            break;
        default:
            break;
    }
    return t;
}

// Bits that must be inside the tile / registers (bit space given by `map`).
uint32_t requirement(const LGate& g, bool backward) {
    switch (g.kind) {
        case K_ROT:
            if (backward && g.grad) return 1u << g.b0;  // the generator pairs amplitudes
            return g.axis == 2 ? 0u : (1u << g.b0);
        case K_U:
            return g.diag ? 0u : (1u << g.b0);
        case K_CNOT:
            return 1u << g.b1;
        case K_SWAP:
            return (1u << g.b0) | (1u << g.b1);
        case K_EMBED:
            return 1u << g.b0;
        default:
            return 0u;
    }
}

int popc(uint32_t x) { return __builtin_popcount(x); }

// Commutation-aware greedy selection.  Walks `pending` in order; a gate is
// placed when it commutes with every gate skipped before it and its required
// bits fit: already in S, or addable (within `addable`, at most `max_add` new
// bits).  `remap` maps global bits of the gate to the selection's bit space.
struct Selector {
    uint32_t S = 0, addable = 0;
    int max_add = 0;
    bool backward = false;
    const int* remap = nullptr;  // nullptr: identity
    int max_grad = 1 << 30;      // gradient-carrying gates per selection (backward tiles)
    // Forward tiles: 2x2 slots per selection.  A run of single-qubit gates on
    // one qubit with nothing else touching it in between becomes one slot;
    // run_open marks the qubits whose last placed touch is such a run.
    int max_mats = 1 << 30;
    uint32_t run_open = 0;

    int m(int b) const { return remap ? remap[b] : b; }

    // Forward: a single-qubit gate that is diagonal in Z (RZ, diagonal U) or
    // in X (RX) and whose next gate on its qubit of another kind (a touch that
    // does not commute with it) is a single-qubit gate is held back and placed
    // together with that gate (right before it), so the two share one 2x2
    // slot -- also across passes: if that gate cannot be placed now, the held
    // one waits with it.  Holding is exact: the held gate commutes with
    // everything between the two (CNOT controls / CZs for Z, CNOT targets for X).
    static int diag_touch_1q(const LGate& g) {
        if ((g.kind == K_ROT && g.axis == 2) || (g.kind == K_U && g.diag)) return T_Z;
        if (g.kind == K_ROT && g.axis == 0) return T_X;
        return -1;
    }
    static bool is_1q(const LGate& g) { return g.kind == K_ROT || g.kind == K_U; }

    std::vector<int> run(const std::vector<int>& pending, const std::vector<LGate>& G) {
        std::vector<int> placed;
        uint32_t sZ = 0, sX = 0, sG = 0;
        std::vector<std::vector<int>> held(32);  // held gates per qubit (pending positions)
        int held_type[32];                        // their touch type (T_Z, T_X or kMixed)
        constexpr int kMixed = -2;
        for (int pi = 0; pi < (int)pending.size(); ++pi) {
            const LGate& g = G[pending[pi]];
            Touch t = touches(g);
            bool ok = true;
            const int dt = backward ? -1 : diag_touch_1q(g);
            const uint32_t blockers = dt == T_Z ? (sX | sG) : (sZ | sG);
            if (dt >= 0 && !(blockers & (1u << m(g.b0)))) {
                // the next gate on the qubit that does not commute with this one
                int next = -1;
                for (int pj = pi + 1; pj < (int)pending.size() && next < 0; ++pj) {
                    const Touch tj = touches(G[pending[pj]]);
                    for (int k = 0; k < tj.count; ++k)
                        if (tj.bit[k] == g.b0 && tj.type[k] != dt) next = pj;
                }
                if (next >= 0 && is_1q(G[pending[next]])) {
                    // a chain of Z- and X-diagonals commutes with no touch of its qubit
                    held_type[g.b0] = held[g.b0].empty() || held_type[g.b0] == dt ? dt : kMixed;
                    held[g.b0].push_back(pi);
                    continue;
                }
            }
            for (int k = 0; k < t.count && ok; ++k) {
                uint32_t bm = 1u << m(t.bit[k]);
                if (t.type[k] == T_Z)
                    ok = !((sX | sG) & bm);
                else if (t.type[k] == T_X)
                    ok = !((sZ | sG) & bm);
                else
                    ok = !((sZ | sX | sG) & bm);
            }
            if (ok && backward && g.grad && max_grad <= 0) ok = false;
            const bool new_mat = !backward && is_1q(g) && !(run_open & (1u << m(g.b0)));
            if (ok && new_mat && max_mats <= 0) ok = false;
            if (ok) {
                uint32_t req = 0;
                uint32_t r = requirement(g, backward);
                // gates released before this one bring their requirements (a held
                // RX needs its qubit in the registers, its partner RZ does not)
                for (int k = 0; k < t.count; ++k)
                    if (t.bit[k] >= 0 && !held[t.bit[k]].empty() && t.type[k] != held_type[t.bit[k]])
                        for (int h : held[t.bit[k]]) r |= requirement(G[pending[h]], backward);
                for (int b = 0; b < 32; ++b)
                    if (r & (1u << b)) req |= 1u << m(b);
                uint32_t nb = req & ~S;
                if (nb == 0) {
                } else if ((nb & ~addable) == 0 && popc(nb) <= max_add) {
                    S |= nb;
                    max_add -= popc(nb);
                } else {
                    ok = false;
                }
                if (ok) {
                    // gates held for this gate go right before it
                    for (int k = 0; k < t.count; ++k)
                        if (t.bit[k] >= 0 && !held[t.bit[k]].empty() && t.type[k] != held_type[t.bit[k]]) {
                            placed.insert(placed.end(), held[t.bit[k]].begin(), held[t.bit[k]].end());
                            held[t.bit[k]].clear();
                        }
                    placed.push_back(pi);
                }
                if (ok && backward && g.grad) --max_grad;
                if (ok && !backward) {
                    if (is_1q(g)) {
                        if (new_mat) --max_mats;
                        run_open |= 1u << m(g.b0);
                    } else {
                        for (int k = 0; k < t.count; ++k)
                            if (t.bit[k] >= 0) run_open &= ~(1u << m(t.bit[k]));
                    }
                }
            }
            if (!ok) {
                for (int k = 0; k < t.count; ++k) {
                    uint32_t bm = 1u << m(t.bit[k]);
                    if (t.type[k] == T_Z) sZ |= bm;
                    else if (t.type[k] == T_X) sX |= bm;
                    else sG |= bm;
                    // gates held for this gate stay pending with it
                    if (t.bit[k] >= 0 && !held[t.bit[k]].empty() && t.type[k] != held_type[t.bit[k]]) {
                        const int ht = held_type[t.bit[k]];
                        if (ht == T_Z) sZ |= bm;
                        else if (ht == T_X) sX |= bm;
                        else sG |= bm;
                        held[t.bit[k]].clear();
                    }
                }
            }
        }
        // (every held diagonal's partner comes later in `pending`, so none is left held)
        return placed;
    }
};

void remove_placed(std::vector<int>& pending, const std::vector<int>& placed_pos) {
    std::vector<char> drop(pending.size(), 0);
    for (int p : placed_pos) drop[p] = 1;
    std::vector<int> rest;
    rest.reserve(pending.size());
    for (size_t i = 0; i < pending.size(); ++i)
        if (!drop[i]) rest.push_back(pending[i]);
    pending.swap(rest);
}

int32_t pack4(const int* v, int count) {
    int32_t r = 0;
    for (int k = 0; k < count; ++k) r |= (v[k] & 15) << (4 * k);
    return r;
}

struct Mapping {
    int reg[5], lane[5], warp[4];
    int nreg, nwarp;
    Mapping() {
        for (int k = 0; k < 5; ++k) reg[k] = lane[k] = -1;
        for (int k = 0; k < 4; ++k) warp[k] = 0;
        nreg = nwarp = 0;
    }
    bool operator==(const Mapping& o) const {
        return !memcmp(reg, o.reg, sizeof(reg)) && !memcmp(lane, o.lane, sizeof(lane)) &&
               !memcmp(warp, o.warp, sizeof(warp)) && nwarp == o.nwarp && nreg == o.nreg;
    }
    void encode(int32_t out[3]) const {
        out[0] = pack4(reg, nreg);
        out[1] = pack4(lane, 5);
        out[2] = pack4(warp, nwarp) | (nwarp << 16);
    }
};

// The mapping used to move a tile between shared memory (natural order) and
// registers: lanes = local bits 0..4 (32 consecutive amplitudes per warp
// access), registers = local bits 5..5+rb-1, warps = the bits above.
Mapping natural_mapping(int tb, int rb) {
    Mapping m;
    m.nreg = rb;
    for (int k = 0; k < 5; ++k) m.lane[k] = k;
    for (int k = 0; k < rb; ++k) m.reg[k] = 5 + k;
    m.nwarp = tb - 5 - rb;
    for (int k = 0; k < m.nwarp; ++k) m.warp[k] = 5 + rb + k;
    return m;
}

// Register set R (local bits) -> full mapping.  Lanes take non-register bits
// whose shared-memory swizzle images are independent (bank-conflict-free
// exchanges); warps take the rest.
Mapping mapping_for(uint32_t R, int tb, int rb) {
    Mapping m;
    m.nreg = rb;
    int r = 0;
    for (int b = 0; b < tb && r < rb; ++b)
        if (R & (1u << b)) m.reg[r++] = b;
    std::vector<int> rest;
    for (int b = 0; b < tb; ++b)
        if (!(R & (1u << b))) rest.push_back(b);
    std::vector<int> lanes;
    // lanes whose bank images (engine.h, bank_image) are linearly independent
    // over GF(2), in ascending local-bit order: kept as a reduced basis
    std::vector<int> basis;
    for (int b : rest) {
        if ((int)lanes.size() >= 5) break;
        int v = qg::bank_image(b);
        for (int e : basis) v = std::min(v, v ^ e);
        if (v) {
            basis.push_back(v);
            lanes.push_back(b);
        }
    }
    for (int b : rest)
        if ((int)lanes.size() < 5 && std::find(lanes.begin(), lanes.end(), b) == lanes.end()) lanes.push_back(b);
    for (int k = 0; k < 5; ++k) m.lane[k] = lanes[k];
    m.nwarp = 0;
    for (int b : rest)
        if (std::find(lanes.begin(), lanes.end(), b) == lanes.end()) m.warp[m.nwarp++] = b;
    return m;
}

struct Slot {
    std::vector<ChainEntry> chain;
    bool per_sample = false;
};

struct PassPlan {
    PassDesc d;
    std::vector<int> gates;  // lowered gate indices in application order
};

}  // namespace

struct Program {
    int n = 0;
    qg_plan_options opt{};
    std::vector<LGate> gates;     // forward order, from the last embedding on
    bool has_embed = false;
    EmbedDesc embed{};
    int nparams = 0, ncols = 0, numats = 0;
    int nsegments = 1;
    std::vector<int> seg_end;     // gate index (exclusive) where each segment ends

    // forward plan
    std::vector<PassDesc> fpass;
    std::vector<int32_t> fops;    // int4 per op
    std::vector<Slot> fslots;
    // backward plan
    std::vector<PassDesc> bpass;
    std::vector<int32_t> bops;
    std::vector<Slot> bslots;
    std::vector<GradTarget> grads;  // per backward grad slot
    // device table layout (byte offsets into the caller's table buffer)
    size_t off_fpass = 0, off_fops = 0, off_fslot = 0, off_fchain = 0;
    size_t off_bpass = 0, off_bops = 0, off_bslot = 0, off_bchain = 0, off_grads = 0, off_embed = 0;
    size_t off_pcsr = 0, off_ccsr = 0;  // per-target lists of grad slots: params, named columns
    std::vector<int32_t> pcsr, ccsr;     // [count + 1] offsets followed by the slot lists
    size_t table_bytes = 0;
    std::vector<unsigned char> table;
    int f_shared = 0, f_ps = 0, b_shared = 0, b_ps = 0;
    std::string stats;
    std::string plan_error;  // set when a pass could not place its gates (the program is refused)
    void* jit = nullptr;  // compiled pass kernels (jit.cpp), owned by the program
};

namespace {

// Emit the device ops of one pass from its placed gates.
// Phase planning: greedily choose register sets; merge runs of single-qubit
// gates on one qubit into one matrix slot (forward only).
// An exchange writes each register to the slot of its logical index, so the
// thread's pending X (register r holds logical amplitude r ^ xm) is folded into
// the write address.  A CNOT whose control is a lane bit makes that pending X
// depend on the lane, and the write's lane -> bank map then carries the bank
// image of the register as well: it can become singular (bank conflicts).
// Walk the pass's ops tracking, per register position, the global bits its
// pending X depends on, and before every exchange whose write map would be
// singular insert OP_XMAT for registers with lane-dependent pending X until
// the map has full rank.
void materialize_before_exchanges(std::vector<int32_t>& ops, const PassDesc& d, int op_begin, int rb) {
    auto rank5 = [](const int v[5]) {
        int basis[5], nb = 0;
        for (int j = 0; j < 5; ++j) {
            int x = v[j];
            for (int e = 0; e < nb; ++e) x = std::min(x, x ^ basis[e]);
            if (x) basis[nb++] = x;
        }
        return nb;
    };
    int reg[5], lane[5];
    auto set_map = [&](int32_t y, int32_t z) {
        for (int k = 0; k < rb; ++k) reg[k] = (y >> (4 * k)) & 15;
        for (int j = 0; j < 5; ++j) lane[j] = (z >> (4 * j)) & 15;
    };
    {
        Mapping nat = natural_mapping(d.tile_bits, rb);
        int32_t e[3];
        nat.encode(e);
        if (d.init == INIT_EMBED) set_map(d.init_map[0], d.init_map[1]);
        else set_map(e[0], e[1]);
    }
    uint32_t form[5] = {0, 0, 0, 0, 0};  // global bits the pending X of each register position depends on
    std::vector<int32_t> out(ops.begin(), ops.begin() + 4 * (size_t)op_begin);
    for (size_t i = 4 * (size_t)op_begin; i < ops.size(); i += 4) {
        const int32_t k = ops[i], y = ops[i + 1], z = ops[i + 2];
        if (k == OP_MAP) {
            uint32_t lane_g = 0;  // global bits of the lanes (qubit bits of the tile only)
            int lg[5];
            for (int j = 0; j < 5; ++j) {
                lg[j] = lane[j] < d.nq_tile ? d.gbit[lane[j]] : -1;
                if (lg[j] >= 0) lane_g |= 1u << lg[j];
            }
            auto write_rank = [&](uint32_t skip) {
                int v[5];
                for (int j = 0; j < 5; ++j) {
                    v[j] = qg::bank_image(lane[j]);
                    if (lg[j] < 0) continue;
                    for (int r = 0; r < rb; ++r)
                        if (!((skip >> r) & 1u) && ((form[r] >> lg[j]) & 1u)) v[j] ^= qg::bank_image(reg[r]);
                }
                return rank5(v);
            };
            while (write_rank(0) < 5) {
                // materialize one register that restores full rank if there is
                // one, else the first with a lane-dependent pending X
                int pick = -1;
                for (int r = 0; r < rb && pick < 0; ++r)
                    if ((form[r] & lane_g) && write_rank(1u << r) == 5) pick = r;
                for (int r = 0; r < rb && pick < 0; ++r)
                    if (form[r] & lane_g) pick = r;
                if (pick < 0) break;  // (cannot happen: without lane-dependent X the map is the lanes')
                out.insert(out.end(), {OP_XMAT, pick, 0, 0});
                form[pick] = 0;
            }
            set_map(y, z);
            for (int r = 0; r < 5; ++r) form[r] = 0;
        } else if (k == OP_CX) {
            if (z & LOC_REG) form[y] ^= form[z & 7];
            else if (z >= 0 && z < 32) form[y] ^= 1u << z;
        } else if (k == OP_SWAP && y != z) {
            std::swap(form[y], form[z]);
        } else if (k == OP_CZ) {
            if (y & LOC_REG) form[y & 7] = 0;
            if (z & LOC_REG) form[z & 7] = 0;
        }
        out.insert(out.end(), ops.begin() + i, ops.begin() + i + 4);
    }
    ops.swap(out);
}

void emit_pass(Program& P, PassPlan& pp, const std::vector<LGate>& G, bool backward,
               std::vector<int32_t>& ops, std::vector<Slot>& slots, int& nshared, int& nps,
               int& nexchanges) {
    PassDesc& d = pp.d;
    const int tb = d.tile_bits;
    // global bit -> local bit
    int g2l[32];
    for (int b = 0; b < 32; ++b) g2l[b] = -1;
    for (int j = 0; j < d.nq_tile; ++j) g2l[d.gbit[j]] = j;
    uint32_t qubit_local = (d.nq_tile >= 32) ? 0xffffffffu : ((1u << d.nq_tile) - 1);

    // the backward holds psi and lambda, so it keeps 16 amplitudes of each per thread
    const int rb = backward ? kBwdRegBits : P.opt.reg_bits;
    Mapping nat = natural_mapping(tb, rb);
    uint32_t natR = 0;
    for (int k = 0; k < rb; ++k) natR |= 1u << nat.reg[k];
    bool nat_ok = (natR & ~qubit_local) == 0;  // natural registers are all qubit bits

    d.op_begin = (int)ops.size() / 4;
    std::vector<int> pending = pp.gates;
    Mapping cur = nat;
    bool have_map = (d.init == INIT_LOAD);  // the load produces the natural mapping
    uint32_t curR = natR;
    bool cur_valid = have_map && nat_ok;
    int first_map_pos = -1;

    auto loc_of = [&](int gbit, const Mapping& mp) -> int32_t {
        int l = g2l[gbit];
        if (l >= 0)
            for (int k = 0; k < rb; ++k)
                if (mp.reg[k] == l) return LOC_REG | k;
        return gbit;
    };
    auto regpos = [&](int gbit, const Mapping& mp) -> int {
        int l = g2l[gbit];
        for (int k = 0; k < rb; ++k)
            if (mp.reg[k] == l) return k;
        return -1;
    };

    // open merge slot per register position (forward): index of op in `ops`
    std::vector<int> open(5, -1);
    auto close_all = [&]() { std::fill(open.begin(), open.end(), -1); };

    int local_remap[32];
    for (int b = 0; b < 32; ++b) local_remap[b] = g2l[b] >= 0 ? g2l[b] : 31;

    while (!pending.empty()) {
        std::vector<int> placed;
        if (cur_valid) {
            Selector s;
            s.S = curR;
            s.addable = 0;
            s.max_add = 0;
            s.backward = backward;
            s.remap = local_remap;
            placed = s.run(pending, G);
        }
        if (placed.empty()) {
            Selector s;
            s.S = 0;
            s.addable = qubit_local;
            s.max_add = rb;
            s.backward = backward;
            s.remap = local_remap;
            placed = s.run(pending, G);
            if (placed.empty()) {
                // the next gate needs bits that are not qubits of this tile:
                // refuse the program rather than loop
                P.plan_error = "a gate does not fit the pass's tile (tile_bits / low_bits leave too few strided qubits)";
                return;
            }
            uint32_t R = s.S;
            // fill to 5 register bits: prefer the natural registers, then low qubit bits
            for (int k = 0; k < rb && popc(R) < rb; ++k)
                if (nat_ok && !(R & (1u << nat.reg[k]))) R |= 1u << nat.reg[k];
            for (int b = 0; b < tb && popc(R) < rb; ++b)
                if ((qubit_local & (1u << b)) && !(R & (1u << b))) R |= 1u << b;
            // Backward plans (and forward plans with reg_search): every register
            // set of rb tile qubits (at most C(13, 5) = 1287) is tried; the one
            // under which the most gates can be placed wins (the greedy set above
            // on ties), so each exchange buys as much work as it can.  Forward
            // plans default to the greedy set: on the 20-qubit forward the search
            // saved 2 of 55 exchanges but ran 1.7 % slower, and serving plans
            // every request; the autotuner times both.
            if ((backward || P.opt.reg_search) && popc(qubit_local) > rb) {
                std::vector<int> qb;
                for (int b = 0; b < tb; ++b)
                    if (qubit_local & (1u << b)) qb.push_back(b);
                const int nq = (int)qb.size();
                size_t best = placed.size();
                for (uint32_t c = (1u << rb) - 1; c < (1u << nq);) {
                    uint32_t C = 0;
                    for (int k = 0; k < nq; ++k)
                        if (c & (1u << k)) C |= 1u << qb[k];
                    Selector t;
                    t.S = C;
                    t.addable = 0;
                    t.max_add = 0;
                    t.backward = backward;
                    t.remap = local_remap;
                    std::vector<int> pl = t.run(pending, G);
                    if (pl.size() > best) {
                        best = pl.size();
                        placed = pl;
                        R = C;
                    }
                    const uint32_t lo = c & (0u - c), hi = c + lo;  // next subset of the same size
                    c = (((hi ^ c) >> 2) / lo) | hi;
                }
            }
            Mapping nm = (R == natR) ? nat : mapping_for(R, tb, rb);
            if (!have_map) {
                // zero / embedding init: produce this mapping directly
                nm.encode(d.init_map);
                have_map = true;
            } else if (!(nm == cur)) {
                int32_t e[3];
                nm.encode(e);
                ops.insert(ops.end(), {OP_MAP, e[0], e[1], e[2]});
                ++nexchanges;
            }
            cur = nm;
            curR = R;
            cur_valid = true;
            close_all();
        }
        (void)first_map_pos;
        // emit placed gates in order
        for (int pi : placed) {
            const LGate& g = G[pending[pi]];
            switch (g.kind) {
                case K_ROT:
                case K_U: {
                    ChainEntry ce{g.kind == K_U ? 3 : g.axis, g.kind == K_U ? 0 : g.src, g.idx,
                                  backward ? 1 : 0};
                    if (g.kind == K_U) ce.src = 0;
                    bool ps = (g.kind == K_ROT && g.src == 1);
                    int rp = regpos(g.b0, cur);
                    if (backward && g.grad) {
                        // gradient partial first, then the inverse gate
                        Slot sl;
                        sl.chain.push_back(ce);
                        sl.per_sample = ps;
                        slots.push_back(sl);
                        int sidx = (int)slots.size() - 1;
                        ops.insert(ops.end(), {OP_MAT, rp, sidx,
                                               (ps ? OPF_PER_SAMPLE : 0) | OPF_GRAD | (g.axis << 8) |
                                                   (g.grad_slot << 12)});
                        break;
                    }
                    bool diag_here = (rp < 0);  // diagonal gate outside the registers
                    int key = diag_here ? -1 : rp;
                    if (!backward && key >= 0 && open[key] >= 0) {
                        int oi = open[key];
                        int sidx = ops[oi + 2];
                        slots[sidx].chain.push_back(ce);
                        if (ps) {
                            slots[sidx].per_sample = true;
                            ops[oi + 3] |= OPF_PER_SAMPLE;
                        }
                        if (ops[oi] == OP_DIAG && !g.diag && !(g.kind == K_ROT && g.axis == 2)) {
                            ops[oi] = OP_MAT;
                            ops[oi + 1] = key;
                        }
                        break;
                    }
                    Slot sl;
                    sl.chain.push_back(ce);
                    sl.per_sample = ps;
                    slots.push_back(sl);
                    int sidx = (int)slots.size() - 1;
                    bool is_diag = g.diag || (g.kind == K_ROT && g.axis == 2);
                    if (is_diag) {
                        int32_t loc = loc_of(g.b0, cur);
                        ops.insert(ops.end(), {OP_DIAG, loc, sidx, ps ? OPF_PER_SAMPLE : 0});
                    } else {
                        ops.insert(ops.end(), {OP_MAT, rp, sidx, ps ? OPF_PER_SAMPLE : 0});
                    }
                    if (key >= 0 && !backward) open[key] = (int)ops.size() - 4;
                    break;
                }
                case K_CNOT: {
                    int rp = regpos(g.b1, cur);
                    int32_t cl = loc_of(g.b0, cur);
                    ops.insert(ops.end(), {OP_CX, rp, cl, 0});
                    if (rp >= 0) open[rp] = -1;
                    if (cl & LOC_REG) open[cl & 7] = -1;
                    break;
                }
                case K_CZ: {
                    int32_t l0 = loc_of(g.b0, cur), l1 = loc_of(g.b1, cur);
                    ops.insert(ops.end(), {OP_CZ, l0, l1, 0});
                    if (l0 & LOC_REG) open[l0 & 7] = -1;
                    if (l1 & LOC_REG) open[l1 & 7] = -1;
                    break;
                }
                case K_SWAP: {
                    int r0 = regpos(g.b0, cur), r1 = regpos(g.b1, cur);
                    ops.insert(ops.end(), {OP_SWAP, r0, r1, 0});
                    open[r0] = -1;
                    open[r1] = -1;
                    break;
                }
                case K_EMBED: {
                    // backward only: gradient of every embedded angle
                    int rp = regpos(g.b0, cur);
                    ops.insert(ops.end(), {OP_GRAD, rp, g.axis, g.grad_slot});
                    break;
                }
            }
        }
        remove_placed(pending, placed);
    }
    if (!have_map) {  // no gate at all: init straight into the natural mapping
        nat.encode(d.init_map);
        have_map = true;
        cur = nat;
    }
    // The epilogue moves the tile through shared memory in natural order.  A
    // forward pass that only stores writes it back from any mapping whose
    // lanes are local bits 0..4 (each warp access still covers consecutive
    // amplitudes), which saves the exchange back to the natural mapping.
    bool need_nat = backward || (d.epi & (EPI_STORE | EPI_PROBS | EPI_P0)) != 0;
    bool lanes_nat = true;
    for (int k = 0; k < 5; ++k) lanes_nat = lanes_nat && cur.lane[k] == k;
    const bool store_only = !backward && (d.epi & (EPI_PROBS | EPI_P0)) == 0;
    if (store_only && lanes_nat) {
        cur.encode(d.end_map);
    } else {
        if (need_nat && !(cur == nat)) {
            int32_t e[3];
            nat.encode(e);
            ops.insert(ops.end(), {OP_MAP, e[0], e[1], e[2]});
            ++nexchanges;
        }
        nat.encode(d.end_map);
    }
    materialize_before_exchanges(ops, d, d.op_begin, rb);
    d.op_count = (int)ops.size() / 4 - d.op_begin;
    (void)nshared;
    (void)nps;
}

// Default cap on the gradient-carrying rotations of a backward pass.  Each
// rotation unrolls into its 2x2 on psi and on lambda and a gradient partial;
// passes of more rotations leave the instruction cache.  Measured on the
// 16-qubit, 20-layer adjoint at batch 1024 (backward ms per step by cap):
// 64 (the shared-memory limit) 48.9, 40 51.6, 36 51.5, 32 42.9, 28 40.0,
// 24 40.7, 16 45.4.
constexpr int kBwdGradPerPass = 28;

// Default cap on the 2x2 slots of a forward pass, for the same reason: the
// compiled pass unrolls every op.  Measured forward ms by cap (uncapped /
// 48 / 32 / 24 / 16): 16 qubits x 1024, 20 layers 10.26 / 10.28 / 8.22 /
// 7.99 / 8.84; 13 qubits x 4096, 20 SEL layers (one pass uncapped) 12.9 /
// 6.54 / 5.85 / 5.22 / 5.43; 28 qubits x 1 156.6 / 156.7 / 153.5 / 154.2 /
// 162.0; the 20-qubit SEL forward already has at most 24 per pass.
constexpr int kFwdMatsPerPass = 24;

// Split a segment of gates into passes (tile selection).
void plan_segment(Program& P, const std::vector<LGate>& G, std::vector<int> pending, int tb,
                  bool backward, std::vector<PassPlan>& out) {
    const int n = P.n;
    // the low run leaves at least two strided slots, so that a two-qubit gate
    // between two strided qubits fits a tile
    const int L = n > tb ? std::min(P.opt.low_bits, tb - 2) : std::min(P.opt.low_bits, std::min(n, tb));
    const int kmax = P.opt.max_high > 0 ? std::min(P.opt.max_high, tb - L) : tb - L;
    while (!pending.empty()) {
        Selector s;
        s.backward = backward;
        if (!backward) s.max_mats = P.opt.fwd_max_mats > 0 ? P.opt.fwd_max_mats : kFwdMatsPerPass;
        if (backward) {
            // gradient-carrying rotations per pass: at most what the kernel's
            // shared memory holds (max_grad_per_pass), by default kBwdGradPerPass
            const int cap = P.opt.bwd_max_grad > 0 ? P.opt.bwd_max_grad : kBwdGradPerPass;
            s.max_grad = std::min(max_grad_per_pass(kBwdRegBits), cap);
        }
        if (n <= tb) {
            s.S = (n >= 32) ? 0xffffffffu : ((1u << n) - 1);
            s.addable = 0;
            s.max_add = 0;
        } else {
            s.S = (1u << L) - 1;
            s.addable = ((n >= 32) ? 0xffffffffu : ((1u << n) - 1)) & ~s.S;
            s.max_add = kmax;
        }
        std::vector<int> placed = s.run(pending, G);
        if (placed.empty()) {
            // cannot happen for valid gates (the first pending gate always fits); guard anyway
            placed.push_back(0);
            uint32_t r = requirement(G[pending[0]], backward);
            s.S |= r;
        }
        PassPlan pp;
        memset(&pp.d, 0, sizeof(pp.d));
        pp.d.tile_bits = tb;
        pp.d.ckpt = -1;
        pp.d.psi_from_ckpt = -1;
        uint32_t S = s.S;
        if (n > tb) {
            for (int b = 0; b < n && popc(S) < tb; ++b) S |= 1u << b;  // fill: extends contiguity
            pp.d.nq_tile = tb;
            int j = 0;
            for (int b = 0; b < n; ++b)
                if (S & (1u << b)) pp.d.gbit[j++] = b;
            int f = 0;
            for (int b = 0; b < n; ++b)
                if (!(S & (1u << b))) pp.d.fixed_gbit[f++] = b;
            pp.d.nfixed = f;
            int run = 0;
            while (run < tb && pp.d.gbit[run] == run) ++run;
            pp.d.run_bits = run;
        } else {
            pp.d.nq_tile = n;
            for (int b = 0; b < n; ++b) pp.d.gbit[b] = b;
            pp.d.nfixed = 0;
            pp.d.run_bits = tb;  // whole samples, consecutive in memory
        }
        for (int pi : placed) pp.gates.push_back(pending[pi]);
        remove_placed(pending, placed);
        out.push_back(pp);
    }
}

void append_slots(std::vector<Slot>& slots, std::vector<SlotDesc>& sd, std::vector<ChainEntry>& ch,
                  int& nshared, int& nps) {
    nshared = nps = 0;
    for (auto& s : slots) {
        SlotDesc d;
        d.chain_begin = (int)ch.size();
        d.chain_len = (int)s.chain.size();
        d.per_sample = s.per_sample ? 1 : 0;
        d.out_index = s.per_sample ? nps++ : nshared++;
        ch.insert(ch.end(), s.chain.begin(), s.chain.end());
        sd.push_back(d);
    }
}

}  // namespace

// Re-number the matrix slot operand of OP_MAT / OP_DIAG to the slot's index
// within its table (shared or per-sample).
static void renumber(std::vector<int32_t>& ops, const std::vector<SlotDesc>& sd) {
    for (size_t i = 0; i < ops.size(); i += 4) {
        if (ops[i] == OP_MAT || ops[i] == OP_DIAG) ops[i + 2] = sd[ops[i + 2]].out_index;
    }
}

static int build_program(Program& P, const qg_gate* gates, int ngates, const int32_t* qlist) {
    const int n = P.n;
    // SWAPs are absorbed by relabelling: perm[b] is the bit of the stored
    // state that holds the reference's bit b.  A SWAP exchanges two entries
    // and emits nothing; every other gate acts on the bits perm points to.
    // At the end, SWAPs on stored bits put every bit back (at most n - 1),
    // so the state, its probabilities and P0 come out in the caller's order.
    int perm[32];
    for (int b = 0; b < 32; ++b) perm[b] = b;
    // the last embedding overwrites the state: everything before it is dead
    int start = 0;
    for (int i = 0; i < ngates; ++i)
        if (gates[i].kind == QG_GATE_EMBED) start = i;
    for (int i = start; i < ngates; ++i) {
        const qg_gate& g = gates[i];
        LGate l;
        switch (g.kind) {
            case QG_GATE_RX:
            case QG_GATE_RY:
            case QG_GATE_RZ:
                if (g.q0 < 0 || g.q0 >= n) return set_error("rotation qubit out of range"), QG_EINVAL;
                if (g.src != 0 && g.src != 1) return set_error("rotation src must be 0 or 1"), QG_EINVAL;
                l.kind = K_ROT;
                l.axis = g.kind;
                l.b0 = perm[n - 1 - g.q0];
                l.src = g.src;
                l.idx = g.idx;
                l.diag = (g.kind == QG_GATE_RZ);
                l.grad = true;
                if (g.src == 0) P.nparams = std::max(P.nparams, g.idx + 1);
                else P.ncols = std::max(P.ncols, g.idx + 1);
                break;
            case QG_GATE_U:
                if (g.q0 < 0 || g.q0 >= n) return set_error("U qubit out of range"), QG_EINVAL;
                l.kind = K_U;
                l.b0 = perm[n - 1 - g.q0];
                l.idx = g.idx;
                l.diag = (g.aux & 1) != 0;  // caller asserts the matrix is diagonal
                P.numats = std::max(P.numats, g.idx + 1);
                break;
            case QG_GATE_CNOT:
            case QG_GATE_CZ:
            case QG_GATE_SWAP:
                if (g.q0 < 0 || g.q0 >= n || g.q1 < 0 || g.q1 >= n)
                    return set_error("two-qubit gate qubit out of range"), QG_EINVAL;
                if (g.q0 == g.q1) {
                    if (g.kind == QG_GATE_SWAP) continue;  // identity (operators.py:661-671)
                    return set_error("control and target must differ"), QG_EINVAL;
                }
                if (g.kind == QG_GATE_SWAP) {
                    std::swap(perm[n - 1 - g.q0], perm[n - 1 - g.q1]);
                    continue;
                }
                l.kind = g.kind == QG_GATE_CNOT ? K_CNOT : K_CZ;
                l.b0 = perm[n - 1 - g.q0];
                l.b1 = perm[n - 1 - g.q1];
                break;
            case QG_GATE_EMBED: {
                if (i != start) break;
                if (g.q0 < 0 || g.q0 > 2) return set_error("embedding axis must be 0..2"), QG_EINVAL;
                if (g.q1 < 0 || g.q1 > 64) return set_error("at most 64 embedded angles"), QG_EINVAL;
                P.has_embed = true;
                P.embed.axis = g.q0;
                P.embed.nq = g.q1;
                P.embed.col0 = g.idx;
                for (int j = 0; j < g.q1; ++j) {
                    int q = qlist[g.aux + j];
                    if (q < 0 || q >= n) return set_error("embedded qubit out of range"), QG_EINVAL;
                    P.embed.qubit[j] = (int8_t)q;
                }
                P.ncols = std::max(P.ncols, g.idx + g.q1);
                continue;
            }
            default:
                return set_error("unknown gate kind"), QG_EINVAL;
        }
        P.gates.push_back(l);
    }
    for (int b = 0; b < n; ++b) {
        if (perm[b] == b) continue;
        int c = 0;
        while (perm[c] != b) ++c;  // the reference bit now stored at bit b
        LGate l;
        l.kind = K_SWAP;
        l.b0 = perm[b];
        l.b1 = b;
        P.gates.push_back(l);
        std::swap(perm[b], perm[c]);
    }
    return QG_OK;
}

static void layout_tables(Program& P) {
    std::vector<SlotDesc> fsd, bsd;
    std::vector<ChainEntry> fch, bch;
    append_slots(P.fslots, fsd, fch, P.f_shared, P.f_ps);
    append_slots(P.bslots, bsd, bch, P.b_shared, P.b_ps);
    renumber(P.fops, fsd);
    renumber(P.bops, bsd);
    auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
    size_t o = 0;
    P.off_fpass = o;
    o = align(o + P.fpass.size() * sizeof(PassDesc));
    P.off_fops = o;
    o = align(o + P.fops.size() * 4);
    P.off_fslot = o;
    o = align(o + fsd.size() * sizeof(SlotDesc));
    P.off_fchain = o;
    o = align(o + fch.size() * sizeof(ChainEntry));
    P.off_bpass = o;
    o = align(o + P.bpass.size() * sizeof(PassDesc));
    P.off_bops = o;
    o = align(o + P.bops.size() * 4);
    P.off_bslot = o;
    o = align(o + bsd.size() * sizeof(SlotDesc));
    P.off_bchain = o;
    o = align(o + bch.size() * sizeof(ChainEntry));
    P.off_grads = o;
    o = align(o + P.grads.size() * sizeof(GradTarget));
    P.off_embed = o;
    o = align(o + sizeof(EmbedDesc));
    // CSR lists: offsets[count + 1] then slots
    auto csr = [&](int src, int count) {
        std::vector<std::vector<int>> lists(count);
        for (size_t gs = 0; gs < P.grads.size(); ++gs)
            if (P.grads[gs].src == src && P.grads[gs].idx < count) lists[P.grads[gs].idx].push_back((int)gs);
        std::vector<int32_t> v(count + 1, 0);
        for (int i = 0; i < count; ++i) v[i + 1] = v[i] + (int)lists[i].size();
        for (auto& l : lists) v.insert(v.end(), l.begin(), l.end());
        return v;
    };
    P.pcsr = csr(0, P.nparams);
    P.ccsr = csr(1, P.ncols);
    P.off_pcsr = o;
    o = align(o + P.pcsr.size() * 4);
    P.off_ccsr = o;
    o = align(o + P.ccsr.size() * 4);
    P.table_bytes = o;
    P.table.assign(o, 0);
    auto put = [&](size_t off, const void* src, size_t bytes) {
        if (bytes) memcpy(P.table.data() + off, src, bytes);
    };
    put(P.off_fpass, P.fpass.data(), P.fpass.size() * sizeof(PassDesc));
    put(P.off_fops, P.fops.data(), P.fops.size() * 4);
    put(P.off_fslot, fsd.data(), fsd.size() * sizeof(SlotDesc));
    put(P.off_fchain, fch.data(), fch.size() * sizeof(ChainEntry));
    put(P.off_bpass, P.bpass.data(), P.bpass.size() * sizeof(PassDesc));
    put(P.off_bops, P.bops.data(), P.bops.size() * 4);
    put(P.off_bslot, bsd.data(), bsd.size() * sizeof(SlotDesc));
    put(P.off_bchain, bch.data(), bch.size() * sizeof(ChainEntry));
    put(P.off_grads, P.grads.data(), P.grads.size() * sizeof(GradTarget));
    put(P.off_embed, &P.embed, sizeof(EmbedDesc));
    put(P.off_pcsr, P.pcsr.data(), P.pcsr.size() * 4);
    put(P.off_ccsr, P.ccsr.data(), P.ccsr.size() * 4);
}

static void plan_forward(Program& P) {
    const int tb = P.opt.tile_bits;
    const int G = (int)P.gates.size();
    int exch = 0;
    std::vector<PassPlan> passes;
    int seg_begin = 0;
    for (int s = 0; s < P.nsegments; ++s) {
        int seg_end = P.seg_end[s];
        std::vector<int> pending;
        for (int i = seg_begin; i < seg_end; ++i) pending.push_back(i);
        size_t before = passes.size();
        plan_segment(P, P.gates, pending, tb, false, passes);
        if (passes.size() == before) {  // empty segment: keep a pass to carry init/epilogue
            PassPlan pp;
            memset(&pp.d, 0, sizeof(pp.d));
            pp.d.tile_bits = tb;
            pp.d.ckpt = -1;
            pp.d.psi_from_ckpt = -1;
            std::vector<PassPlan> tmp;
            plan_segment(P, P.gates, {}, tb, false, tmp);
            int n = P.n;
            if (n > tb) {
                pp.d.nq_tile = tb;
                for (int j = 0; j < tb; ++j) pp.d.gbit[j] = j;
                for (int b = tb; b < n; ++b) pp.d.fixed_gbit[b - tb] = b;
                pp.d.nfixed = n - tb;
                pp.d.run_bits = tb;
            } else {
                pp.d.nq_tile = n;
                for (int b = 0; b < n; ++b) pp.d.gbit[b] = b;
                pp.d.run_bits = tb;
            }
            passes.push_back(pp);
        }
        if (s + 1 < P.nsegments) passes.back().d.ckpt = s;  // state at the segment end
        seg_begin = seg_end;
    }
    (void)G;
    const int m = P.opt.measure;
    for (size_t p = 0; p < passes.size(); ++p) {
        PassDesc& d = passes[p].d;
        d.init = (p == 0) ? (P.has_embed ? INIT_EMBED : INIT_LOAD) : INIT_LOAD;
        bool last = (p + 1 == passes.size());
        int epi = EPI_STORE;
        if (last) {
            epi = 0;
            if (m == QG_MEASURE_STATE || m == QG_MEASURE_NONE || P.opt.keep_state) epi |= EPI_STORE;
            if (m == QG_MEASURE_PROBS) epi |= EPI_PROBS;
            if (m == QG_MEASURE_P0 || m == QG_MEASURE_Z) epi |= EPI_P0;
        }
        d.epi = epi;
        emit_pass(P, passes[p], P.gates, false, P.fops, P.fslots, P.f_shared, P.f_ps, exch);
        P.fpass.push_back(d);
    }
    P.stats = "forward: " + std::to_string(P.fpass.size()) + " passes, " +
              std::to_string(P.fops.size() / 4) + " ops, " + std::to_string(exch) + " exchanges";
}

static void plan_backward(Program& P) {
    const int tb = P.opt.tile_bits - 1;  // psi and lambda tiles share the shared memory
    // reversed gate list; rotations carry a gradient
    std::vector<LGate> rev;
    for (int i = (int)P.gates.size() - 1; i >= 0; --i) {
        LGate g = P.gates[i];
        g.grad = (g.kind == K_ROT);
        rev.push_back(g);
    }
    // embedding: a gradient-only op per embedded angle, at the very end
    if (P.has_embed) {
        for (int j = 0; j < P.embed.nq; ++j) {
            LGate g;
            g.kind = K_EMBED;
            g.axis = P.embed.axis;
            g.b0 = P.n - 1 - P.embed.qubit[j];
            g.grad = true;
            g.src = 1;
            g.idx = P.embed.col0 + j;
            rev.push_back(g);
        }
    }
    int exch = 0;
    std::vector<PassPlan> passes;
    // segments in reverse; the backward of segment s starts from its checkpoint
    const int G = (int)P.gates.size();
    int total = (int)rev.size();
    int seg_hi = G;  // forward index (exclusive) of the current segment's end
    int rpos = 0;
    for (int s = P.nsegments - 1; s >= 0; --s) {
        int seg_lo = s == 0 ? 0 : P.seg_end[s - 1];
        int count = seg_hi - seg_lo;
        std::vector<int> pending;
        for (int k = 0; k < count; ++k) pending.push_back(rpos + k);
        if (s == 0)
            for (int k = count; rpos + k < total; ++k) pending.push_back(rpos + k);  // embedding grads
        size_t before = passes.size();
        plan_segment(P, rev, pending, tb, true, passes);
        if (s + 1 < P.nsegments && passes.size() > before) passes[before].d.psi_from_ckpt = s;
        rpos += count;
        seg_hi = seg_lo;
    }
    // gradient slots in pass order: each pass owns a contiguous range
    P.grads.clear();
    for (auto& pp : passes)
        for (int gi : pp.gates)
            if (rev[gi].grad) {
                rev[gi].grad_slot = (int)P.grads.size();
                P.grads.push_back(GradTarget{rev[gi].src, rev[gi].idx});
            }
    for (size_t p = 0; p < passes.size(); ++p) {
        PassDesc& d = passes[p].d;
        d.init = INIT_LOAD;
        // the final backward pass stores lambda only when the caller asks for
        // the input-state gradient (a launch flag); it still ends in the
        // natural mapping so that store is possible
        d.epi = (p + 1 == passes.size()) ? 0 : EPI_STORE;
        emit_pass(P, passes[p], rev, true, P.bops, P.bslots, P.b_shared, P.b_ps, exch);
        // grad slots of this pass
        int lo = 1 << 30, hi = -1;
        for (size_t i = d.op_begin * 4; i < P.bops.size(); i += 4) {
            int32_t opc = P.bops[i];
            int gs = -1;
            if (opc == OP_MAT && (P.bops[i + 3] & OPF_GRAD)) gs = P.bops[i + 3] >> 12;
            if (opc == OP_GRAD) gs = P.bops[i + 3];
            if (gs >= 0) lo = std::min(lo, gs), hi = std::max(hi, gs);
        }
        d.grad_base = hi >= 0 ? lo : 0;
        d.ngrad = hi >= 0 ? hi - lo + 1 : 0;
        P.bpass.push_back(d);
    }
    P.stats += "; backward: " + std::to_string(P.bpass.size()) + " passes, " +
               std::to_string(P.bops.size() / 4) + " ops, " + std::to_string(exch) + " exchanges";
}

void program_run_info(const void* prog, ProgramRun* r) {
    const Program& P = *reinterpret_cast<const Program*>(prog);
    r->n = P.n;
    r->tile_bits = P.opt.tile_bits;
    r->reg_bits = P.opt.reg_bits;
    r->measure = P.opt.measure;
    r->keep_state = P.opt.keep_state;
    r->segments = P.nsegments;
    r->nparams = P.nparams;
    r->ncols = P.ncols;
    r->numats = P.numats;
    r->ngrads = (int)P.grads.size();
    r->has_embed = P.has_embed ? 1 : 0;
    r->nfslots = (int)P.fslots.size();
    r->f_shared = P.f_shared;
    r->f_ps = P.f_ps;
    r->nbslots = (int)P.bslots.size();
    r->b_shared = P.b_shared;
    r->b_ps = P.b_ps;
    r->nfpass = (int)P.fpass.size();
    r->nbpass = (int)P.bpass.size();
    r->fpass = P.fpass.data();
    r->bpass = P.bpass.data();
    r->fops = P.fops.data();
    r->bops = P.bops.data();
    r->off_fpass = P.off_fpass;
    r->off_fops = P.off_fops;
    r->off_fslot = P.off_fslot;
    r->off_fchain = P.off_fchain;
    r->off_bpass = P.off_bpass;
    r->off_bops = P.off_bops;
    r->off_bslot = P.off_bslot;
    r->off_bchain = P.off_bchain;
    r->off_embed = P.off_embed;
    r->off_pcsr = P.off_pcsr;
    r->off_ccsr = P.off_ccsr;
}

void* program_jit_state(const void* prog) { return reinterpret_cast<const Program*>(prog)->jit; }
void program_set_jit_state(void* prog, void* state) { reinterpret_cast<Program*>(prog)->jit = state; }

}  // namespace qg

using qg::Program;

extern "C" {

void qg_plan_options_default(qg_plan_options* o) {
    memset(o, 0, sizeof(*o));
    o->tile_bits = 13;
    o->low_bits = 6;
    o->max_high = 0;
    o->measure = QG_MEASURE_STATE;
    o->keep_state = 0;
    o->segments = 1;
    o->reg_bits = 5;
}

int qg_program_create(const qg_gate* gates, int ngates, const int32_t* qlist, int n,
                      const qg_plan_options* opt, qg_program** out) {
    if (!out) return qg::set_error("out is null"), QG_EINVAL;
    *out = nullptr;
    if (n < 5 || n > qg::kMaxQubits)
        return qg::set_error("the fused engine needs 5 <= num_qubits <= 30"), QG_EINVAL;
    if (ngates < 0 || (ngates > 0 && !gates)) return qg::set_error("bad gate list"), QG_EINVAL;
    qg_plan_options o;
    if (opt) o = *opt;
    else qg_plan_options_default(&o);
    if (o.tile_bits < 11 || o.tile_bits > qg::kMaxTileBits)
        return qg::set_error("tile_bits must be in [11, 13]"), QG_EINVAL;
    if (o.low_bits < 4 || o.low_bits > o.tile_bits - 1)
        return qg::set_error("low_bits must be in [4, tile_bits - 1]"), QG_EINVAL;
    if (o.max_high < 0) return qg::set_error("max_high must be >= 0"), QG_EINVAL;
    if (o.reg_bits != 4 && o.reg_bits != 5) return qg::set_error("reg_bits must be 4 or 5"), QG_EINVAL;
    if (o.tile_bits - 5 - o.reg_bits < 0 || o.tile_bits - 5 - o.reg_bits > 4)
        return qg::set_error("tile_bits - reg_bits must leave 0..4 warp bits"), QG_EINVAL;
    if (o.segments < 1) o.segments = 1;
    if (o.reg_search != 0 && o.reg_search != 1) return qg::set_error("reg_search must be 0 or 1"), QG_EINVAL;
    if (o.bwd_max_grad < 0) return qg::set_error("bwd_max_grad must be >= 0"), QG_EINVAL;
    if (o.fwd_max_mats < 0) return qg::set_error("fwd_max_mats must be >= 0"), QG_EINVAL;
    std::unique_ptr<Program> P(new Program());
    P->n = n;
    P->opt = o;
    int rc = qg::build_program(*P, gates, ngates, qlist);
    if (rc) return rc;
    const int G = (int)P->gates.size();
    P->nsegments = std::max(1, std::min(o.segments, std::max(1, G)));
    for (int s = 1; s <= P->nsegments; ++s) P->seg_end.push_back((int)((int64_t)G * s / P->nsegments));
    qg::plan_forward(*P);
    qg::plan_backward(*P);
    if (!P->plan_error.empty()) return qg::set_error("qg_program_create: " + P->plan_error), QG_EINVAL;
    qg::layout_tables(*P);
    *out = reinterpret_cast<qg_program*>(P.release());
    return QG_OK;
}

void qg_program_destroy(qg_program* p) {
    if (!p) return;
    Program* P = reinterpret_cast<Program*>(p);
    qg::jit_release(P->jit);
    delete P;
}

int qg_program_info(const qg_program* p, qg_program_info_t* info) {
    if (!p || !info) return qg::set_error("null pointer"), QG_EINVAL;
    const Program& P = *reinterpret_cast<const Program*>(p);
    memset(info, 0, sizeof(*info));
    info->num_qubits = P.n;
    info->forward_passes = (int)P.fpass.size();
    info->backward_passes = (int)P.bpass.size();
    info->forward_ops = (int)P.fops.size() / 4;
    info->backward_ops = (int)P.bops.size() / 4;
    info->gates = (int)P.gates.size();
    info->nparams = P.nparams;
    info->ncols = P.ncols;
    info->numats = P.numats;
    info->grad_slots = (int)P.grads.size();
    info->forward_shared_slots = P.f_shared;
    info->forward_sample_slots = P.f_ps;
    info->backward_shared_slots = P.b_shared;
    info->backward_sample_slots = P.b_ps;
    info->segments = P.nsegments;
    info->table_bytes = (int64_t)P.table_bytes;
    info->has_embedding = P.has_embed ? 1 : 0;
    snprintf(info->summary, sizeof(info->summary), "%s", P.stats.c_str());
    return QG_OK;
}

int qg_program_table(const qg_program* p, void* host_out, int64_t bytes) {
    if (!p || !host_out) return qg::set_error("null pointer"), QG_EINVAL;
    const Program& P = *reinterpret_cast<const Program*>(p);
    if (bytes < (int64_t)P.table_bytes) return qg::set_error("table buffer too small"), QG_ENOMEM;
    memcpy(host_out, P.table.data(), P.table_bytes);
    return QG_OK;
}

int qg_program_pass(const qg_program* p, int backward, int index, qg_pass_info_t* out) {
    if (!p || !out) return qg::set_error("null pointer"), QG_EINVAL;
    const Program& P = *reinterpret_cast<const Program*>(p);
    const std::vector<qg::PassDesc>& v = backward ? P.bpass : P.fpass;
    const std::vector<int32_t>& ops = backward ? P.bops : P.fops;
    if (index < 0 || index >= (int)v.size()) return qg::set_error("pass index out of range"), QG_EINVAL;
    const qg::PassDesc& d = v[index];
    memset(out, 0, sizeof(*out));
    out->tile_bits = d.tile_bits;
    out->nq_tile = d.nq_tile;
    out->run_bits = d.run_bits;
    out->nfixed = d.nfixed;
    for (int j = 0; j < 16; ++j) out->gbit[j] = d.gbit[j];
    for (int j = 0; j < 32; ++j) out->fixed_gbit[j] = d.fixed_gbit[j];
    out->op_count = d.op_count;
    out->init = d.init;
    out->epi = d.epi;
    for (int k = 0; k < 3; ++k) out->init_map[k] = d.init_map[k];
    out->ckpt = d.ckpt;
    out->psi_from_ckpt = d.psi_from_ckpt;
    out->grad_base = d.grad_base;
    out->ngrad = d.ngrad;
    out->ops = ops.data() + 4 * (size_t)d.op_begin;
    return QG_OK;
}

int qg_program_grad_targets(const qg_program* p, int32_t* out, int64_t cap) {
    if (!p) return qg::set_error("null pointer"), -1;
    const Program& P = *reinterpret_cast<const Program*>(p);
    int count = (int)P.grads.size();
    if (out && cap >= 2 * (int64_t)count)
        for (int i = 0; i < count; ++i) out[2 * i] = P.grads[i].src, out[2 * i + 1] = P.grads[i].idx;
    return count;
}

int qg_program_slots(const qg_program* p, int backward, int32_t* out, int64_t cap) {
    if (!p) return qg::set_error("null pointer"), -1;
    const Program& P = *reinterpret_cast<const Program*>(p);
    const std::vector<qg::Slot>& slots = backward ? P.bslots : P.fslots;
    std::vector<int32_t> v;
    int nshared = 0, nps = 0;
    for (const auto& s : slots) {
        v.push_back(s.per_sample ? 1 : 0);
        v.push_back(s.per_sample ? nps++ : nshared++);
        v.push_back((int32_t)s.chain.size());
        for (const auto& c : s.chain) v.insert(v.end(), {c.kind, c.src, c.idx, c.dagger});
    }
    if (out && cap >= (int64_t)v.size()) memcpy(out, v.data(), v.size() * 4);
    return (int)v.size();
}

}  // extern "C"

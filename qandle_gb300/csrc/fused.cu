// Fused form: shared-memory-staged passes that apply many gates per HBM round
// trip, and the adjoint backward over the same program.
//
// One persistent CTA per SM walks the tiles of a pass.  A tile is 2^TB
// amplitudes (TB = 13 forward, 12 backward) spanning TB qubits of one sample,
// or whole samples when n < TB.  Its memory image is contiguous blocks of at
// least 2^run_bits amplitudes; producer warps move them between global memory
// and a ring of shared-memory tile buffers with bulk (TMA) copies, so later
// tiles stream in and earlier ones stream out while the compute warps work on
// the current one.  Compute threads hold 2^RB amplitudes each in registers;
// gates act in registers, and an OP_MAP exchange through a swizzled
// shared-memory layout changes which tile qubits are register qubits.  The
// forward kernel body lives in fwd_kernel.cuh; this file holds its op
// interpreter, the backward kernel, the helper kernels and the host side.
//
// The gate programs come from the planner in program.cpp.  The rotation and
// matrix algebra follows the reference's row-vector convention,
// out = in @ M (qandle/operators.py:265-298, :368-395, :125-126).
#include <cuda_runtime.h>

#include <cstring>
#include <type_traits>

#include "common.cuh"
#include "engine.h"
#include "bwd_kernel.cuh"
#include "fwd_kernel.cuh"
#include "jit.h"
#include "planar.cuh"
#include "qandle_gb300.h"

namespace qg {

// Run f(integral_constant<P>) for the runtime register position p < RB.
template <int RB, typename F>
__device__ __forceinline__ void for_pos(int p, F&& f) {
    switch (p) {
        case 0: f(std::integral_constant<int, 0>{}); break;
        case 1: f(std::integral_constant<int, 1>{}); break;
        case 2: f(std::integral_constant<int, 2>{}); break;
        case 3: f(std::integral_constant<int, 3>{}); break;
        default:
            if constexpr (RB > 4) f(std::integral_constant<int, 4>{});
            break;
    }
}

// Apply the pending X of register bit p to the given tiles and clear it.
template <int RB, int NTILE>
__device__ __forceinline__ void pmaterialize(PTile<RB>* const (&ts)[NTILE], uint32_t& xm, int p) {
    const bool c = (xm >> p) & 1;
#pragma unroll
    for (int i = 0; i < NTILE; ++i)
        for_pos<RB>(p, [&](auto P) { pswap_if<decltype(P)::value, RB>(*ts[i], c); });
    xm &= ~(1u << p);
}

template <int RB>
__device__ __forceinline__ void pnegate_mask(PTile<RB>& t, uint32_t mask) {
    // mask has 0, 1 or 2 register bits
    switch (mask) {
        case 0: pnegate<0, RB>(t); break;
        case 1: pnegate<1, RB>(t); break;
        case 2: pnegate<2, RB>(t); break;
        case 4: pnegate<4, RB>(t); break;
        case 8: pnegate<8, RB>(t); break;
        case 3: pnegate<3, RB>(t); break;
        case 5: pnegate<5, RB>(t); break;
        case 6: pnegate<6, RB>(t); break;
        case 9: pnegate<9, RB>(t); break;
        case 10: pnegate<10, RB>(t); break;
        case 12: pnegate<12, RB>(t); break;
        default:
            if constexpr (RB > 4) {
                switch (mask) {
                    case 16: pnegate<16, RB>(t); break;
                    case 17: pnegate<17, RB>(t); break;
                    case 18: pnegate<18, RB>(t); break;
                    case 20: pnegate<20, RB>(t); break;
                    case 24: pnegate<24, RB>(t); break;
                    default: break;
                }
            }
            break;
    }
}

// Apply one non-map op to NTILE planar tiles (psi, and lambda in the
// backward) that share the pending X mask xm.
template <int RB, int NTILE>
__device__ __forceinline__ void papply_op(const int4 op, PTile<RB>* const (&ts)[NTILE], uint32_t& xm,
                                          const ThreadMap& tm, const RunArgs& A, const float4* smats,
                                          int64_t sample) {
    switch (op.x) {
        case OP_MAT: {
            float2 m[4];
            load_slot(A, smats, op.z, op.w, sample, m);
            if ((xm >> op.y) & 1) {  // X M X
                const float2 m0 = m[0], m1 = m[1];
                m[0] = m[3];
                m[1] = m[2];
                m[2] = m1;
                m[3] = m0;
            }
#pragma unroll
            for (int i = 0; i < NTILE; ++i)
                for_pos<RB>(op.y, [&](auto P) { pmat<decltype(P)::value, RB>(*ts[i], m); });
            break;
        }
        case OP_DIAG: {
            float2 m[4];
            load_slot(A, smats, op.z, op.w, sample, m);
            if (op.y & LOC_REG) {
                const int p = op.y & 7;
                const bool sw = (xm >> p) & 1;
                const float2 d0 = sw ? m[3] : m[0], d1 = sw ? m[0] : m[3];
#pragma unroll
                for (int i = 0; i < NTILE; ++i)
                    for_pos<RB>(p, [&](auto P) { pdiag<decltype(P)::value, RB>(*ts[i], d0, d1); });
            } else {
                const float2 d = loc_bit_thread(op.y, tm.tglob) ? m[3] : m[0];
#pragma unroll
                for (int i = 0; i < NTILE; ++i) pscale<RB>(*ts[i], d);
            }
            break;
        }
        case OP_CX: {
            if (op.z & LOC_REG) {
                const int c = op.z & 7;
                // the same rules as the compiled passes' jcx, so that both
                // kernels apply every later 2x2 to the same operands in the
                // same order: the register CNOT runs on the physical bits and
                // a pending X on the control stays pending (X_c CX X_c = X_t
                // CX: it moves a pending X onto the target); a pending X on
                // the target commutes with the CNOT
#pragma unroll
                for (int i = 0; i < NTILE; ++i)
                    for_pos<RB>(op.y, [&](auto P) {
                        for_pos<RB>(c, [&](auto C) {
                            if constexpr (decltype(P)::value != decltype(C)::value)
                                pcx<decltype(P)::value, decltype(C)::value, RB>(*ts[i]);
                        });
                    });
                xm ^= ((xm >> c) & 1u) << op.y;
            } else {
                xm ^= (uint32_t)loc_bit_thread(op.z, tm.tglob) << op.y;
            }
            break;
        }
        case OP_CZ: {
            uint32_t mask = 0;
            bool cond = true;
            if (op.y & LOC_REG) {
                const int p = op.y & 7;
                if ((xm >> p) & 1) pmaterialize<RB, NTILE>(ts, xm, p);
                mask |= 1u << p;
            } else {
                cond = cond && loc_bit_thread(op.y, tm.tglob);
            }
            if (op.z & LOC_REG) {
                const int p = op.z & 7;
                if ((xm >> p) & 1) pmaterialize<RB, NTILE>(ts, xm, p);
                mask |= 1u << p;
            } else {
                cond = cond && loc_bit_thread(op.z, tm.tglob);
            }
            if (cond)
#pragma unroll
                for (int i = 0; i < NTILE; ++i) pnegate_mask<RB>(*ts[i], mask);
            break;
        }
        case OP_XMAT:
            pmaterialize<RB, NTILE>(ts, xm, op.y);
            break;
        case OP_SWAP: {
            if (op.y == op.z) break;
            // as the compiled passes' jswap: swap the physical bits and their
            // pending X flags
#pragma unroll
            for (int i = 0; i < NTILE; ++i)
                for_pos<RB>(op.y, [&](auto P0) {
                    for_pos<RB>(op.z, [&](auto P1) {
                        if constexpr (decltype(P0)::value != decltype(P1)::value)
                            pswapbits<decltype(P0)::value, decltype(P1)::value, RB>(*ts[i]);
                    });
                });
            const uint32_t dx = ((xm >> op.y) ^ (xm >> op.z)) & 1u;
            xm ^= dx * ((1u << op.y) | (1u << op.z));
            break;
        }
        default:
            break;
    }
}

// Gradient partial on register bit p with the pending X folded in: the
// physical pair order turns the generator G into X G X (= -G for Y and Z).
template <int RB>
__device__ __forceinline__ float pgrad_op(const PTile<RB>& ps, const PTile<RB>& ls, int p, int axis, uint32_t xm) {
    float g = 0.f;
    for_pos<RB>(p, [&](auto P) { g = pgrad<decltype(P)::value, RB>(ps, ls, axis); });
    return (((xm >> p) & 1) && axis != AX_X) ? -g : g;
}

// --------------------------------------------- the op interpreter --

// Gate program of a forward pass read from the pass's op list at run time
// (the prebuilt kernels; the compiled pass kernels of jit.cpp unroll it).
struct InterpOps {
    static constexpr bool kStageOps = true;
    // init, epilogue and end mapping come from the pass descriptor at run time
    static constexpr int kInit = -1;
    static constexpr int kEpi = -1;
    static constexpr int kEndNatural = -1;
    static constexpr uint32_t kStagedBytes = 0;
    __device__ __forceinline__ static void stage(const RunArgs&, const TileGeo&, float4*, uint64_t*, int) {}
    template <int TB, int RB>
    __device__ __forceinline__ static void apply(PTile<RB>& pt, uint32_t& xm, ThreadMap& tm, const PassDesc& d,
                                                 const RunArgs& A, const int4* ops, const int4* s_ops,
                                                 const float4* s_mats, float* plane, int64_t sample0,
                                                 uint32_t fixed_val, int tid) {
        for (int o = 0; o < d.op_count; ++o) {
            int4 op = o < kSmemOps ? s_ops[o] : __ldg(ops + o);
            if (op.x == OP_MAP) {
                exchange<TB, RB>(pt, xm, tm, plane, d, op.y, op.z, op.w, tid, fixed_val);
            } else {
                PTile<RB>* const tiles[1] = {&pt};
                papply_op<RB, 1>(op, tiles, xm, tm, A, s_mats, sample0 + tm.sample_off);
            }
        }
    }
};

template <int TB, int RB, int MAXJ>
__global__ void __launch_bounds__(fwd_threads(TB, RB), fwd_min_blocks(TB, RB))
    k_fwd_pass(const __grid_constant__ JobTable<MAXJ> jt) {
    fwd_pass_body<TB, RB, MAXJ, InterpOps>(jt);
}

// Gate program of a backward pass read from the pass's op list at run time.
struct BwdInterpOps {
    static constexpr bool kStageOps = true;
    template <int TB, int RB>
    __device__ __forceinline__ static void apply(PTile<RB>& pt, PTile<RB>& lt, uint32_t& xm, ThreadMap& tm,
                                                 const PassDesc& d, const RunArgs& A, const int4* ops,
                                                 const int4* s_ops, const float4* s_mats, float* pp, float* lp,
                                                 int64_t sample0, uint32_t fixed_val, int tid, float* gacc,
                                                 uint8_t* gsmp) {
        constexpr int NT = 1 << (TB - RB);
        PTile<RB>* const tiles[2] = {&pt, &lt};
        for (int o = 0; o < d.op_count; ++o) {
            int4 op = o < kSmemOps ? s_ops[o] : __ldg(ops + o);
            if (op.x == OP_MAP) {
                exchange2<TB, RB>(pt, lt, xm, tm, pp, lp, d, op.y, op.z, op.w, tid, fixed_val);
            } else if (op.x == OP_GRAD) {
                grad_record<NT>(gacc, gsmp, op.w - d.grad_base, tid, pgrad_op<RB>(pt, lt, op.y, op.z, xm),
                                tm.sample_off);
            } else if (op.x == OP_MAT && (op.w & OPF_GRAD)) {
                const int axis = (op.w >> 8) & 3;
                const int gslot = op.w >> 12;
                grad_record<NT>(gacc, gsmp, gslot - d.grad_base, tid, pgrad_op<RB>(pt, lt, op.y, axis, xm),
                                tm.sample_off);
                papply_op<RB, 2>(make_int4(OP_MAT, op.y, op.z, op.w), tiles, xm, tm, A, s_mats,
                                 sample0 + tm.sample_off);
            } else {
                papply_op<RB, 2>(op, tiles, xm, tm, A, s_mats, sample0 + tm.sample_off);
            }
        }
    }
};

template <int TB, int RB>
__global__ void __launch_bounds__(bwd_threads(TB, RB), 1)
    k_bwd_pass(const PassDesc* __restrict__ passes, const int4* __restrict__ ops_all, int pass_index, RunArgs A,
               int store_lam_last, int64_t num_tiles) {
    bwd_pass_body<TB, RB, BwdInterpOps>(passes, ops_all, pass_index, A, store_lam_last, num_tiles);
}

// ------------------------------------------------------------ helpers --

// Build the matrix tables: product of each slot's chain in row form.
__global__ void k_build_mats(const SlotDesc* __restrict__ slots, const ChainEntry* __restrict__ chain, int nslots,
                             int nshared, int nps, int64_t batch, const float* __restrict__ params,
                             const float* __restrict__ named, int ncols, const float2* __restrict__ umats,
                             float2* __restrict__ mats, float2* __restrict__ mats_ps) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    // items: shared slots once, per-sample slots once per sample
    int64_t total = (int64_t)nslots * 1;  // slot index space
    (void)total;
    int64_t s_items = nshared;
    int64_t p_items = (int64_t)nps * batch;
    if (i >= s_items + p_items) return;
    int slot_index;
    int64_t b = 0;
    bool per_sample;
    if (i < s_items) {
        slot_index = (int)i;
        per_sample = false;
    } else {
        int64_t k = i - s_items;
        b = k / nps;
        slot_index = (int)(k % nps);
        per_sample = true;
    }
    // find the slot with this out_index (slots are few; linear scan is fine)
    const SlotDesc* sd = nullptr;
    for (int s = 0; s < nslots; ++s)
        if (slots[s].per_sample == (per_sample ? 1 : 0) && slots[s].out_index == slot_index) {
            sd = &slots[s];
            break;
        }
    if (!sd) return;
    float2 m[4] = {make_float2(1.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(1.f, 0.f)};
    for (int c = 0; c < sd->chain_len; ++c) {
        ChainEntry e = chain[sd->chain_begin + c];
        float2 g[4];
        if (e.kind == 3) {
            g[0] = umats[4 * e.idx];
            g[1] = umats[4 * e.idx + 1];
            g[2] = umats[4 * e.idx + 2];
            g[3] = umats[4 * e.idx + 3];
        } else {
            float th = e.src == 0 ? params[e.idx] : named[b * ncols + e.idx];
            rotation_row_matrix(e.kind, th, g);
        }
        if (e.dagger) dagger_row_matrix(g);
        // m = m @ g
        float2 r0 = cadd(cmul(m[0], g[0]), cmul(m[1], g[2]));
        float2 r1 = cadd(cmul(m[0], g[1]), cmul(m[1], g[3]));
        float2 r2 = cadd(cmul(m[2], g[0]), cmul(m[3], g[2]));
        float2 r3 = cadd(cmul(m[2], g[1]), cmul(m[3], g[3]));
        m[0] = r0;
        m[1] = r1;
        m[2] = r2;
        m[3] = r3;
    }
    float2* dst = per_sample ? mats_ps + (b * nps + slot_index) * 4 : mats + (int64_t)slot_index * 4;
    dst[0] = m[0];
    dst[1] = m[1];
    dst[2] = m[2];
    dst[3] = m[3];
}

// Embedding factors R(x)|0> per sample and qubit; unlisted qubits keep |0>.
__global__ void k_embed_fac(const EmbedDesc* __restrict__ ed, const float* __restrict__ named, int ncols,
                            int64_t batch, int n, float2* __restrict__ fac) {
    int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= batch) return;
    EmbedDesc e = *ed;
    float2* f = fac + b * n * 2;
    for (int q = 0; q < n; ++q) {
        f[2 * q] = make_float2(1.f, 0.f);
        f[2 * q + 1] = make_float2(0.f, 0.f);
    }
    for (int j = 0; j < e.nq; ++j) {
        int q = e.qubit[j];
        float2 m[4];
        rotation_row_matrix(e.axis, named[b * ncols + e.col0 + j], m);
        float2 v0 = f[2 * q], v1 = f[2 * q + 1];
        f[2 * q] = cadd(cmul(m[0], v0), cmul(m[2], v1));
        f[2 * q + 1] = cadd(cmul(m[1], v0), cmul(m[3], v1));
    }
}

// P0 / <Z> from the last pass's tile partials, in double, in tile order.
__global__ void k_p0_finalize(const PassDesc* __restrict__ last, const float* __restrict__ part, float* out,
                              int64_t batch, int n, int tb, int z) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= batch * n) return;
    const PassDesc& d = *last;
    int64_t b = i / n;
    int q = (int)(i % n);
    int gb = n - 1 - q;
    int local = -1, fixed_k = -1;
    for (int j = 0; j < d.nq_tile; ++j)
        if (d.gbit[j] == gb) local = j;
    for (int k = 0; k < d.nfixed; ++k)
        if (d.fixed_gbit[k] == gb) fixed_k = k;
    int64_t tps = (n >= tb) ? (int64_t(1) << (n - tb)) : 1;
    const float* p = part + b * tps * (tb + 1);
    double p0 = 0.0, tot = 0.0;
    for (int64_t t = 0; t < tps; ++t) {
        const float* row = p + t * (tb + 1);
        tot += row[tb];
        if (local >= 0)
            p0 += row[local];
        else if (fixed_k >= 0 && !((t >> fixed_k) & 1))
            p0 += row[tb];
    }
    out[i] = z ? (float)(2.0 * p0 - tot) : (float)p0;
}

// lambda = dL/dpsi* from the upstream gradient of the measured output.
__global__ void k_seed(const float2* __restrict__ psi, const void* __restrict__ gout, float2* __restrict__ lam,
                       int64_t total, int n, int measure) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= total) return;
    float2 a = psi[i];
    if (measure == QG_MEASURE_P0 || measure == QG_MEASURE_Z) {
        int64_t b = i >> n;
        uint32_t k = (uint32_t)(i & ((int64_t(1) << n) - 1));
        const float* g = reinterpret_cast<const float*>(gout) + b * n;
        float w = 0.f;
        for (int q = 0; q < n; ++q) {
            bool zero = !((k >> (n - 1 - q)) & 1);
            w += measure == QG_MEASURE_Z ? (zero ? g[q] : -g[q]) : (zero ? g[q] : 0.f);
        }
        lam[i] = make_float2(w * a.x, w * a.y);
    } else if (measure == QG_MEASURE_PROBS) {
        float w = reinterpret_cast<const float*>(gout)[i];
        lam[i] = make_float2(w * a.x, w * a.y);
    } else {
        float2 g = reinterpret_cast<const float2*>(gout)[i];
        lam[i] = make_float2(0.5f * g.x, 0.5f * g.y);
    }
}

// Reduce gradient partials per target in double, in a fixed order.
__global__ void k_grad_finalize(const int32_t* __restrict__ pcsr, int nparams, const int32_t* __restrict__ ccsr,
                                int ncols, const float* __restrict__ part, int64_t units, int64_t batch,
                                int64_t tps, float* __restrict__ dparams, float* __restrict__ dnamed) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < nparams) {
        double acc = 0.0;
        for (int k = pcsr[i]; k < pcsr[i + 1]; ++k) {
            int gs = pcsr[nparams + 1 + k];
            const float* p = part + (int64_t)gs * units;
            for (int64_t u = 0; u < units; ++u) acc += p[u];
        }
        if (dparams) dparams[i] = (float)acc;
        return;
    }
    i -= nparams;
    if (i >= (int64_t)ncols * batch) return;
    int64_t b = i / ncols;
    int c = (int)(i % ncols);
    double acc = 0.0;
    for (int k = ccsr[c]; k < ccsr[c + 1]; ++k) {
        int gs = ccsr[ncols + 1 + k];
        const float* p = part + (int64_t)gs * units + b * tps;
        for (int64_t u = 0; u < tps; ++u) acc += p[u];
    }
    if (dnamed) dnamed[b * ncols + c] = (float)acc;
}

__global__ void k_scale2(const float2* __restrict__ lam, float2* __restrict__ out, int64_t total) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < total) out[i] = make_float2(2.f * lam[i].x, 2.f * lam[i].y);
}

}  // namespace qg

// ---------------------------------------------------------- host side --

namespace qg {

static int sm_count() {
    static int cached = 0;
    if (!cached) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev);
        if (cached <= 0) cached = 1;
    }
    return cached;
}

static size_t al(size_t x) { return (x + 255) & ~size_t(255); }

struct FwdLayout {
    size_t status, mats, mats_ps, embfac, p0part, total;
};
struct BwdLayout {
    size_t status, mats, mats_ps, gradpart, total;
    int64_t units, tps;
};

static FwdLayout fwd_layout(const ProgramRun& R, int64_t B) {
    FwdLayout L;
    size_t o = 0;
    L.status = o;
    o = al(o + 16);
    L.mats = o;
    o = al(o + (size_t)R.f_shared * 32);
    L.mats_ps = o;
    o = al(o + (size_t)B * R.f_ps * 32);
    L.embfac = o;
    o = al(o + (R.has_embed ? (size_t)B * R.n * 16 : 0));
    L.p0part = o;
    int tb = R.tile_bits;
    int64_t tps = R.n >= tb ? (int64_t(1) << (R.n - tb)) : 1;
    bool p0 = R.measure == QG_MEASURE_P0 || R.measure == QG_MEASURE_Z;
    o = al(o + (p0 ? (size_t)B * tps * (tb + 1) * 4 : 0));
    L.total = o;
    return L;
}

static BwdLayout bwd_layout(const ProgramRun& R, int64_t B) {
    BwdLayout L;
    size_t o = 0;
    L.status = o;
    o = al(o + 16);
    L.mats = o;
    o = al(o + (size_t)R.b_shared * 32);
    L.mats_ps = o;
    o = al(o + (size_t)B * R.b_ps * 32);
    int tb = R.tile_bits - 1;
    L.tps = R.n >= tb ? (int64_t(1) << (R.n - tb)) : 1;
    L.units = R.n >= tb ? B * L.tps : B;
    L.gradpart = o;
    o = al(o + (size_t)R.ngrads * L.units * 4);
    L.total = o;
    return L;
}

template <int TB, int RB, int MAXJ>
static int launch_fwd_jobs(const JobTable<MAXJ>& jt, cudaStream_t st) {
    constexpr int NT = fwd_threads(TB, RB);
    size_t smem = fwd_smem_bytes(TB);
    static bool attr_set = false;
    if (!attr_set) {
        QG_CUDA_TRY(
            cudaFuncSetAttribute(k_fwd_pass<TB, RB, MAXJ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = true;
    }
    int64_t tiles = jt.begin[jt.njobs];
    if (tiles <= 0) return QG_OK;
    static int per_sm = 0;
    if (!per_sm) {
        QG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fwd_pass<TB, RB, MAXJ>, NT, smem));
        if (per_sm < 1) per_sm = 1;
    }
    int64_t slots = (int64_t)sm_count() * per_sm;  // persistent: every resident CTA walks tiles
    int64_t grid = tiles < slots ? tiles : slots;
    k_fwd_pass<TB, RB, MAXJ><<<(unsigned)grid, NT, smem, st>>>(jt);
    QG_LAUNCH_CHECK();
    return QG_OK;
}

// Launch a job table on the kernel instantiated for (tile_bits, reg_bits).
static int launch_fwd_table(const JobTable<QG_MAX_JOBS>& jt, int tb, int rb, cudaStream_t st) {
    if (rb == 4) {
        switch (tb) {
            case 13: return launch_fwd_jobs<13, 4, QG_MAX_JOBS>(jt, st);
            case 12: return launch_fwd_jobs<12, 4, QG_MAX_JOBS>(jt, st);
            default: return launch_fwd_jobs<11, 4, QG_MAX_JOBS>(jt, st);
        }
    }
    switch (tb) {
        case 13: return launch_fwd_jobs<13, 5, QG_MAX_JOBS>(jt, st);
        case 12: return launch_fwd_jobs<12, 5, QG_MAX_JOBS>(jt, st);
        default: return launch_fwd_jobs<11, 5, QG_MAX_JOBS>(jt, st);
    }
}

static int launch_fwd_pass(const PassDesc* dpass, const int4* dops, const PassDesc& hpass, int p, const RunArgs& A,
                           int zero_init, int64_t tiles, int tb, int rb, cudaStream_t st) {
    static thread_local JobTable<QG_MAX_JOBS> jt;  // host staging; copied into the launch parameters
    memset(&jt, 0, sizeof(jt));
    jt.njobs = 1;
    jt.begin[0] = 0;
    jt.begin[1] = tiles;
    jt.job[0].pd = dpass + p;
    jt.job[0].ops = dops + hpass.op_begin;
    jt.job[0].A = A;
    jt.job[0].zero_init = zero_init;
    jt.job[0].tiles = tiles;
    return launch_fwd_table(jt, tb, rb, st);
}

// One-job launch of a pass kernel compiled for this program (jit.cpp).
static int launch_fwd_compiled(const JitKernel& k, const PassDesc* dpass, const int4* dops, const PassDesc& hpass,
                               int p, const RunArgs& A, int zero_init, int64_t tiles, int rb, cudaStream_t st) {
    JobTable<1> jt;
    memset(&jt, 0, sizeof(jt));
    jt.njobs = 1;
    jt.begin[0] = 0;
    jt.begin[1] = tiles;
    jt.job[0].pd = dpass + p;
    jt.job[0].ops = dops + hpass.op_begin;
    jt.job[0].A = A;
    jt.job[0].zero_init = zero_init;
    jt.job[0].tiles = tiles;
    if (tiles <= 0) return QG_OK;
    const int tb = hpass.tile_bits;
    int64_t slots = (int64_t)sm_count() * k.per_sm;
    int64_t grid = tiles < slots ? tiles : slots;
    void* params[] = {&jt};
    return jit_launch(k, (unsigned)grid, (unsigned)fwd_threads(tb, rb), (size_t)fwd_smem_bytes(tb), st, params);
}

template <int TB, int RB>
static int launch_bwd_pass(const PassDesc* dpass, const int4* dops, int p, const RunArgs& A, int store_lam,
                           int64_t tiles, cudaStream_t st) {
    constexpr int NT = bwd_threads(TB, RB);
    size_t smem = bwd_smem_bytes(TB, RB);
    static bool attr_set = false;
    if (!attr_set) {
        QG_CUDA_TRY(cudaFuncSetAttribute(k_bwd_pass<TB, RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = true;
    }
    static int per_sm = 0;
    if (!per_sm) {
        QG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bwd_pass<TB, RB>, NT, smem));
        if (per_sm < 1) per_sm = 1;
    }
    int64_t slots = (int64_t)sm_count() * per_sm;
    int64_t grid = tiles < slots ? tiles : slots;
    k_bwd_pass<TB, RB><<<(unsigned)grid, NT, smem, st>>>(dpass, dops, p, A, store_lam, tiles);
    QG_LAUNCH_CHECK();
    return QG_OK;
}

// Launch of a backward pass kernel compiled for this program (jit.cpp).
static int launch_bwd_compiled(const JitKernel& k, const PassDesc* dpass, const int4* dops, int p, const RunArgs& A,
                               int store_lam, int64_t tiles, int tb, cudaStream_t st) {
    if (tiles <= 0) return QG_OK;
    const int rb = kBwdRegBits;
    int64_t slots = (int64_t)sm_count() * k.per_sm;
    int64_t grid = tiles < slots ? tiles : slots;
    RunArgs a = A;
    int pass = p, sl = store_lam;
    int64_t nt = tiles;
    void* params[] = {(void*)&dpass, (void*)&dops, &pass, &a, &sl, &nt};
    return jit_launch(k, (unsigned)grid, (unsigned)bwd_threads(tb, rb), (size_t)bwd_smem_bytes(tb, rb), st, params);
}

static int launch_bwd(const PassDesc* dpass, const int4* dops, int p, const RunArgs& A, int store_lam,
                      int64_t tiles, int tb, int rb, cudaStream_t st) {
    static_assert(kBwdRegBits == 4, "backward kernels are instantiated for 4 register bits");
    (void)rb;
    switch (tb) {
        case 12: return launch_bwd_pass<12, 4>(dpass, dops, p, A, store_lam, tiles, st);
        case 11: return launch_bwd_pass<11, 4>(dpass, dops, p, A, store_lam, tiles, st);
        default: return launch_bwd_pass<10, 4>(dpass, dops, p, A, store_lam, tiles, st);
    }
}

// A wait that runs out on purpose: one CTA waits on an mbarrier nothing
// arrives on, with a short limit, and reports what the bounded wait saw.
__global__ void k_selftest_wait(int* status, uint64_t limit_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const bool done = mbar_wait(&bar, 0, limit_ns);
    if (threadIdx.x == 0) *status = done ? 0 : kStatusTimeout;
}

// FP32 roof probe: every thread runs 8 independent chains of packed FMAs
// (fma.rn.f32x2, 2 FMAs per instruction) and its block writes one sum, so
// nothing is dead code.  Four 256-thread blocks per SM keep 8 warps on each
// scheduler.  b < 1 and c small keep the values finite.
constexpr int kProbeChains = 8;
__global__ void __launch_bounds__(256) k_fp32_probe(float* out, int64_t iters) {
    float2 a[kProbeChains];
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) a[k] = make_float2(1e-3f * (threadIdx.x + k), 1e-3f * k);
    const float2 b = make_float2(0.999999f, 0.999998f), c = make_float2(1e-7f, 2e-7f);
    for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kProbeChains; ++k) a[k] = vfma(a[k], b, c);
    }
    float v = 0.f;
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) v += a[k].x + a[k].y;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __shared__ float part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < 8; ++w) t += part[w];
        out[blockIdx.x] = t;
    }
}

static int64_t num_tiles(int n, int tb, int64_t B) {
    if (n >= tb) return B << (n - tb);
    int64_t spt = int64_t(1) << (tb - n);
    return (B + spt - 1) / spt;
}

}  // namespace qg

extern "C" {

int64_t qg_program_workspace_bytes(const qg_program* prog, int64_t batch, int backward) {
    if (!prog || batch < 1) return -1;
    qg::ProgramRun R;
    qg::program_run_info(prog, &R);
    return backward ? (int64_t)qg::bwd_layout(R, batch).total : (int64_t)qg::fwd_layout(R, batch).total;
}

int qg_program_forward(const qg_program* prog, const void* dev_table, void* workspace, int64_t workspace_bytes,
                       void* state, int64_t batch, int zero_init, const float* params, const float* named,
                       const void* umats, float* out, void* ckpt, void* stream) {
    return qg_program_forward_timed(prog, dev_table, workspace, workspace_bytes, state, batch, zero_init, params,
                                    named, umats, out, ckpt, nullptr, stream);
}

static int fwd_args(const qg_program* prog, const void* dev_table, void* workspace, int64_t workspace_bytes,
                    void* state, int64_t batch, float* out, void* ckpt, qg::ProgramRun& R, qg::RunArgs& A,
                    qg::FwdLayout& L) {
    using namespace qg;
    QG_CHECK_ARG(prog && dev_table && workspace && state, "null pointer");
    QG_CHECK_ARG(batch >= 1, "batch must be >= 1");
    QG_CHECK_ARG(((uintptr_t)state & 15) == 0, "state must be 16-byte aligned");
    program_run_info(prog, &R);
    L = fwd_layout(R, batch);
    QG_CHECK_ARG(workspace_bytes >= (int64_t)L.total, "workspace too small");
    bool p0 = R.measure == QG_MEASURE_P0 || R.measure == QG_MEASURE_Z;
    QG_CHECK_ARG(!(p0 || R.measure == QG_MEASURE_PROBS) || out, "out is null");
    QG_CHECK_ARG(!out || ((uintptr_t)out & 15) == 0, "out must be 16-byte aligned");
    char* ws = (char*)workspace;
    A = RunArgs{};
    A.state = (float2*)state;
    A.ckpt = (float2*)ckpt;
    A.out = out;
    A.p0part = (float*)(ws + L.p0part);
    A.mats = (const float2*)(ws + L.mats);
    A.mats_ps = (const float2*)(ws + L.mats_ps);
    A.embfac = (const float2*)(ws + L.embfac);
    A.status = (int*)(ws + L.status);
    A.batch = batch;
    A.n = R.n;
    A.nslots_ps = R.f_ps;
    A.nslots_shared = R.f_shared;
    return QG_OK;
}

int qg_program_prepare(const qg_program* prog, const void* dev_table, void* workspace, int64_t workspace_bytes,
                       int64_t batch, const float* params, const float* named, const void* umats, void* stream) {
    using namespace qg;
    QG_CHECK_ARG(prog && dev_table && workspace, "null pointer");
    QG_CHECK_ARG(batch >= 1, "batch must be >= 1");
    ProgramRun R;
    program_run_info(prog, &R);
    FwdLayout L = fwd_layout(R, batch);
    QG_CHECK_ARG(workspace_bytes >= (int64_t)L.total, "workspace too small");
    QG_CHECK_ARG(R.nparams == 0 || params, "params is null");
    QG_CHECK_ARG(R.ncols == 0 || named, "named inputs are null");
    QG_CHECK_ARG(R.numats == 0 || umats, "umats is null");
    cudaStream_t st = (cudaStream_t)stream;
    char* ws = (char*)workspace;
    const char* tab = (const char*)dev_table;
    QG_CUDA_TRY(cudaMemsetAsync(ws + L.status, 0, 16, st));
    int64_t items = R.f_shared + (int64_t)R.f_ps * batch;
    if (items > 0) {
        k_build_mats<<<grid_for(items, 128), 128, 0, st>>>(
            (const SlotDesc*)(tab + R.off_fslot), (const ChainEntry*)(tab + R.off_fchain), R.nfslots, R.f_shared,
            R.f_ps, batch, params, named, R.ncols, (const float2*)umats, (float2*)(ws + L.mats),
            (float2*)(ws + L.mats_ps));
        QG_LAUNCH_CHECK();
    }
    if (R.has_embed) {
        k_embed_fac<<<grid_for(batch, 128), 128, 0, st>>>((const EmbedDesc*)(tab + R.off_embed), named, R.ncols,
                                                         batch, R.n, (float2*)(ws + L.embfac));
        QG_LAUNCH_CHECK();
    }
    return QG_OK;
}

int qg_program_finish(const qg_program* prog, const void* dev_table, void* workspace, int64_t workspace_bytes,
                      int64_t batch, float* out, void* stream) {
    using namespace qg;
    QG_CHECK_ARG(prog && dev_table && workspace, "null pointer");
    ProgramRun R;
    program_run_info(prog, &R);
    FwdLayout L = fwd_layout(R, batch);
    QG_CHECK_ARG(workspace_bytes >= (int64_t)L.total, "workspace too small");
    bool p0 = R.measure == QG_MEASURE_P0 || R.measure == QG_MEASURE_Z;
    if (!p0) return QG_OK;
    QG_CHECK_ARG(out, "out is null");
    const PassDesc* dpass = (const PassDesc*)((const char*)dev_table + R.off_fpass);
    k_p0_finalize<<<grid_for(batch * R.n, 128), 128, 0, (cudaStream_t)stream>>>(
        dpass + (R.nfpass - 1), (const float*)((char*)workspace + L.p0part), out, batch, R.n, R.tile_bits,
        R.measure == QG_MEASURE_Z);
    QG_LAUNCH_CHECK();
    return QG_OK;
}

int qg_workspace_status(const void* workspace, void* stream) {
    QG_CHECK_ARG(workspace, "null pointer");
    int h[4] = {0, 0, 0, 0};  // status, wait site, block, tile
    cudaStream_t st = (cudaStream_t)stream;
    QG_CUDA_TRY(cudaMemcpyAsync(h, workspace, sizeof(h), cudaMemcpyDeviceToHost, st));
    QG_CUDA_TRY(cudaStreamSynchronize(st));
    if (h[0] == 0) return QG_OK;
    qg::set_error(h[0] == QG_ETIMEOUT
                      ? "a kernel wait timed out (a producer / compute hand-off never completed): wait site " +
                            std::to_string(h[1]) + ", block " + std::to_string(h[2]) + ", tile " +
                            std::to_string(h[3])
                      : "a kernel reported an error status");
    return h[0];
}

int64_t qg_fp32_probe_blocks(void) { return (int64_t)qg::sm_count() * 4; }

int qg_fp32_probe(float* out, int64_t out_floats, int64_t iters, int64_t* fma_count, void* stream) {
    const int64_t blocks = qg_fp32_probe_blocks();
    QG_CHECK_ARG(out && fma_count, "null pointer");
    QG_CHECK_ARG(blocks > 0 && out_floats >= blocks, "out holds fewer floats than qg_fp32_probe_blocks()");
    QG_CHECK_ARG(iters >= 1 && iters <= (int64_t(1) << 24), "iters must be in [1, 2^24]");
    qg::k_fp32_probe<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(out, iters);
    QG_LAUNCH_CHECK();
    *fma_count = blocks * 256 * iters * qg::kProbeChains * 2;
    return QG_OK;
}

int qg_selftest_wait_timeout(int64_t limit_ns, void* stream) {
    QG_CHECK_ARG(limit_ns > 0 && limit_ns <= 2000000000LL, "limit_ns must be in (0, 2e9]");
    cudaStream_t st = (cudaStream_t)stream;
    int* d = nullptr;
    QG_CUDA_TRY(cudaMalloc(&d, sizeof(int)));
    int h = -1;
    cudaError_t e = cudaMemsetAsync(d, 0xff, sizeof(int), st);
    if (e == cudaSuccess) {
        qg::k_selftest_wait<<<1, 32, 0, st>>>(d, (uint64_t)limit_ns);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d);
    if (e != cudaSuccess) return qg::set_error(std::string("selftest: ") + cudaGetErrorString(e)), QG_ECUDA;
    if (h == QG_ETIMEOUT) return QG_ETIMEOUT;
    return qg::set_error("selftest: the wait did not report a timeout"), QG_ECUDA;
}

int qg_jobs_run_pass(const qg_job* jobs, int njobs, void* stream) {
    using namespace qg;
    QG_CHECK_ARG(njobs >= 0 && njobs <= QG_MAX_JOBS, "njobs must be in [0, 32]");
    QG_CHECK_ARG(njobs == 0 || jobs, "jobs is null");
    if (njobs == 0) return QG_OK;
    static thread_local JobTable<QG_MAX_JOBS> jt;  // host staging of the launch parameters
    memset(&jt, 0, sizeof(jt));
    int tb = -1, rb = 5;
    int64_t acc = 0;
    for (int i = 0; i < njobs; ++i) {
        const qg_job& q = jobs[i];
        ProgramRun R;
        RunArgs A;
        FwdLayout L;
        int rc = fwd_args(q.prog, q.table, q.workspace, q.workspace_bytes, q.state, q.batch, q.out, nullptr, R, A, L);
        if (rc) return rc;
        QG_CHECK_ARG(q.pass >= 0 && q.pass < R.nfpass, "pass index out of range");
        QG_CHECK_ARG(R.segments <= 1, "checkpointed programs run through qg_program_forward");
        if (tb < 0) tb = R.tile_bits, rb = R.reg_bits;
        QG_CHECK_ARG(tb == R.tile_bits && rb == R.reg_bits,
                     "all jobs of one launch need the same tile_bits and reg_bits");
        const char* tab = (const char*)q.table;
        jt.job[i].pd = (const PassDesc*)(tab + R.off_fpass) + q.pass;
        jt.job[i].ops = (const int4*)(tab + R.off_fops) + R.fpass[q.pass].op_begin;
        jt.job[i].A = A;
        jt.job[i].zero_init = (q.pass == 0) ? q.zero_init : 0;
        jt.job[i].tiles = num_tiles(R.n, R.tile_bits, q.batch);
        jt.begin[i] = acc;
        acc += jt.job[i].tiles;
    }
    jt.njobs = njobs;
    jt.begin[njobs] = acc;
    return launch_fwd_table(jt, tb, rb, (cudaStream_t)stream);
}

int qg_job_run_pass_compiled(const qg_job* job, void* stream) {
    using namespace qg;
    QG_CHECK_ARG(job, "job is null");
    ProgramRun R;
    RunArgs A;
    FwdLayout L;
    int rc = fwd_args(job->prog, job->table, job->workspace, job->workspace_bytes, job->state, job->batch, job->out,
                      nullptr, R, A, L);
    if (rc) return rc;
    QG_CHECK_ARG(job->pass >= 0 && job->pass < R.nfpass, "pass index out of range");
    QG_CHECK_ARG(R.segments <= 1, "checkpointed programs run through qg_program_forward");
    JitKernel jk;
    QG_CHECK_ARG(jit_forward_kernel(job->prog, job->pass, &jk),
                 "the program's pass kernels are not compiled for the current device (qg_program_compile)");
    const char* tab = (const char*)job->table;
    return launch_fwd_compiled(jk, (const PassDesc*)(tab + R.off_fpass), (const int4*)(tab + R.off_fops),
                               R.fpass[job->pass], job->pass, A, job->pass == 0 ? job->zero_init : 0,
                               num_tiles(R.n, R.tile_bits, job->batch), R.reg_bits, (cudaStream_t)stream);
}

int qg_program_forward_timed(const qg_program* prog, const void* dev_table, void* workspace,
                             int64_t workspace_bytes, void* state, int64_t batch, int zero_init, const float* params,
                             const float* named, const void* umats, float* out, void* ckpt,
                             void* const* pass_events, void* stream) {
    using namespace qg;
    ProgramRun R;
    RunArgs A;
    FwdLayout L;
    int rc = fwd_args(prog, dev_table, workspace, workspace_bytes, state, batch, out, ckpt, R, A, L);
    if (rc) return rc;
    QG_CHECK_ARG(R.segments <= 1 || ckpt, "checkpoint buffer is null");
    rc = qg_program_prepare(prog, dev_table, workspace, workspace_bytes, batch, params, named, umats, stream);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const char* tab = (const char*)dev_table;
    const PassDesc* dpass = (const PassDesc*)(tab + R.off_fpass);
    const int4* dops = (const int4*)(tab + R.off_fops);
    int64_t tiles = num_tiles(R.n, R.tile_bits, batch);
    for (int p = 0; p < R.nfpass; ++p) {
        int zi = (p == 0) ? zero_init : 0;
        if (pass_events) QG_CUDA_TRY(cudaEventRecord((cudaEvent_t)pass_events[2 * p], st));
        JitKernel jk;
        if (jit_forward_kernel(prog, p, &jk))
            rc = launch_fwd_compiled(jk, dpass, dops, R.fpass[p], p, A, zi, tiles, R.reg_bits, st);
        else
            rc = launch_fwd_pass(dpass, dops, R.fpass[p], p, A, zi, tiles, R.tile_bits, R.reg_bits, st);
        if (rc) return rc;
        if (pass_events) QG_CUDA_TRY(cudaEventRecord((cudaEvent_t)pass_events[2 * p + 1], st));
    }
    return qg_program_finish(prog, dev_table, workspace, workspace_bytes, batch, out, stream);
}

int qg_program_backward(const qg_program* prog, const void* dev_table, void* workspace, int64_t workspace_bytes,
                        void* state, void* lam, int64_t batch, const float* params, const float* named,
                        const void* umats, const void* grad_out, float* dparams, float* dnamed, void* dstate,
                        const void* ckpt, void* stream) {
    return qg_program_backward_timed(prog, dev_table, workspace, workspace_bytes, state, lam, batch, params, named,
                                     umats, grad_out, dparams, dnamed, dstate, ckpt, nullptr, stream);
}

int qg_program_backward_timed(const qg_program* prog, const void* dev_table, void* workspace,
                              int64_t workspace_bytes, void* state, void* lam, int64_t batch, const float* params,
                              const float* named, const void* umats, const void* grad_out, float* dparams,
                              float* dnamed, void* dstate, const void* ckpt, void* const* pass_events,
                              void* stream) {
    using namespace qg;
    QG_CHECK_ARG(prog && dev_table && workspace && state && lam && grad_out, "null pointer");
    QG_CHECK_ARG(batch >= 1, "batch must be >= 1");
    QG_CHECK_ARG(((uintptr_t)state & 15) == 0 && ((uintptr_t)lam & 15) == 0, "state / lam must be 16-byte aligned");
    ProgramRun R;
    program_run_info(prog, &R);
    BwdLayout L = bwd_layout(R, batch);
    QG_CHECK_ARG(workspace_bytes >= (int64_t)L.total, "workspace too small");
    QG_CHECK_ARG(R.segments <= 1 || ckpt, "checkpoint buffer is null");
    cudaStream_t st = (cudaStream_t)stream;
    char* ws = (char*)workspace;
    const char* tab = (const char*)dev_table;
    RunArgs A{};
    A.state = (float2*)state;
    A.lam = (float2*)lam;
    A.ckpt = (float2*)ckpt;
    A.gradpart = (float*)(ws + L.gradpart);
    A.mats = (const float2*)(ws + L.mats);
    A.mats_ps = (const float2*)(ws + L.mats_ps);
    A.status = (int*)(ws + L.status);
    A.batch = batch;
    A.n = R.n;
    A.nslots_ps = R.b_ps;
    A.nslots_shared = R.b_shared;
    QG_CUDA_TRY(cudaMemsetAsync(ws + L.status, 0, 16, st));
    int64_t items = R.b_shared + (int64_t)R.b_ps * batch;
    if (items > 0) {
        k_build_mats<<<grid_for(items, 128), 128, 0, st>>>(
            (const SlotDesc*)(tab + R.off_bslot), (const ChainEntry*)(tab + R.off_bchain), R.nbslots, R.b_shared,
            R.b_ps, batch, params, named, R.ncols, (const float2*)umats, (float2*)(ws + L.mats),
            (float2*)(ws + L.mats_ps));
        QG_LAUNCH_CHECK();
    }
    int64_t total = batch << R.n;
    k_seed<<<grid_for(total, 256), 256, 0, st>>>((const float2*)state, grad_out, (float2*)lam, total, R.n,
                                                 R.measure);
    QG_LAUNCH_CHECK();
    if (R.ngrads > 0) QG_CUDA_TRY(cudaMemsetAsync(A.gradpart, 0, (size_t)R.ngrads * L.units * 4, st));
    const PassDesc* dpass = (const PassDesc*)(tab + R.off_bpass);
    const int4* dops = (const int4*)(tab + R.off_bops);
    int tb = R.tile_bits - 1;
    int64_t tiles = num_tiles(R.n, tb, batch);
    for (int p = 0; p < R.nbpass; ++p) {
        int store_lam = (p + 1 == R.nbpass) && dstate != nullptr;
        if (pass_events) QG_CUDA_TRY(cudaEventRecord((cudaEvent_t)pass_events[2 * p], st));
        JitKernel jk;
        int rc = jit_backward_kernel(prog, p, &jk)
                     ? launch_bwd_compiled(jk, dpass, dops, p, A, store_lam, tiles, tb, st)
                     : launch_bwd(dpass, dops, p, A, store_lam, tiles, tb, kBwdRegBits, st);
        if (rc) return rc;
        if (pass_events) QG_CUDA_TRY(cudaEventRecord((cudaEvent_t)pass_events[2 * p + 1], st));
    }
    int64_t fitems = R.nparams + (int64_t)R.ncols * batch;
    if (fitems > 0) {
        k_grad_finalize<<<grid_for(fitems, 128), 128, 0, st>>>(
            (const int32_t*)(tab + R.off_pcsr), R.nparams, (const int32_t*)(tab + R.off_ccsr), R.ncols, A.gradpart,
            L.units, batch, (R.n >= tb ? L.tps : 1), dparams, dnamed);
        QG_LAUNCH_CHECK();
    }
    if (dstate) {
        k_scale2<<<grid_for(total, 256), 256, 0, st>>>((const float2*)lam, (float2*)dstate, total);
        QG_LAUNCH_CHECK();
    }
    return QG_OK;
}

}  // extern "C"

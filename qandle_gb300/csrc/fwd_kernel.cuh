// Forward pass kernel shared by the prebuilt op interpreter (fused.cu) and
// by the pass kernels the library compiles at run time with NVRTC for one
// program (jit.cpp).  Everything here is device code that needs no host
// header, so the same text is handed to NVRTC.
//
// A pass walks tiles of 2^TB amplitudes through a ring of three shared-memory
// buffers.  Producer warps move the tiles with bulk (TMA) copies: they load
// tile t+1 and store tile t-2 while the compute warps work on tile t,
// and the two sides hand buffers over through a full and an empty mbarrier per
// buffer.  A compute thread holds 2^RB amplitudes in registers
// (planar.cuh); the gate program of the pass runs on them (`Ops`), exchanging
// through the tile's buffer when the register qubits change; the epilogue
// writes the tile back into its buffer and computes its probabilities or P0
// partials.
#pragma once
#include "devmath.cuh"
#include "engine.h"
#include "planar.cuh"

namespace qg {

// ------------------------------------------------------------------ PTX --

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void bulk_s2g(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read0() {
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---------------------------------------------- producer / compute sync --

// Compute-warp barrier (named barrier 1): the producer warps of a forward CTA
// never join it.  In a backward CTA, N is the whole block.
template <int N>
__device__ __forceinline__ void cta_sync() {
    asm volatile("bar.sync 1, %0;" ::"n"(N) : "memory");
}
// cta_sync that also ANDs a flag over the N threads.
template <int N>
__device__ __forceinline__ bool cta_sync_and(bool v) {
    uint32_t r;
    asm volatile(
        "{ .reg .pred p, q; setp.ne.u32 p, %1, 0; bar.red.and.pred q, 1, %2, p; selp.u32 %0, 1, 0, q; }"
        : "=r"(r)
        : "r"((uint32_t)v), "n"(N)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void mbar_init(uint64_t* b, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("{ .reg .b64 st; mbarrier.arrive.shared::cta.b64 st, [%0]; }" ::"r"(smem_u32(b)) : "memory");
}
// Test for the completion of the phase of parity `parity`; a waiting thread
// is suspended (up to about a millisecond) instead of polling shared memory.
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3; selp.b32 %0, 1, 0, p; }"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity), "r"(1000000u)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait for the phase of parity `parity` of b.  False when it did not
// complete within limit_ns (about two seconds by default; at most 2^16
// tries): the caller reports kStatusTimeout and winds the CTA down instead of
// waiting on.
constexpr uint64_t kWaitNs = 2000000000ull;
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, uint64_t limit_ns = kWaitNs) {
    if (mbar_try_wait(b, parity)) return true;
    const uint64_t t0 = global_ns();
    // the time limit ends the wait; the try count is a second bound in case
    // the timer stalls (a try may return at once instead of suspending, so the
    // count is set high enough never to end a wait before the time limit)
    for (uint32_t i = 1; i < (1u << 26); ++i) {
        if (mbar_try_wait(b, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
    return false;
}

// Where a bounded wait gave up, recorded next to the status word (the
// workspace's first 16 bytes: status, site, block, tile) by the first CTA
// that reports a timeout.
enum WaitSite : int {
    kSiteFwdProducer = 1,  // forward producer, waiting for a buffer to be released
    kSiteFwdCompute = 2,   // forward compute warps, waiting for a tile to land
    kSiteBwdProducer = 5,  // backward producer / compute warps
    kSiteBwdCompute = 6,
};
__device__ __forceinline__ void report_timeout(int* status, int site, int64_t tile) {
    if (atomicExch(status, kStatusTimeout) == 0) {
        status[1] = site;
        status[2] = (int)blockIdx.x;
        status[3] = (int)tile;
    }
}

// ------------------------------------------------------- tile geometry --

// Swizzled shared-memory slot of local index j in an exchange plane (see
// swz_slot in engine.h: the bank bits take the XOR of the images of the high
// bits, so lanes whose local bits have independent images hit 32 distinct
// banks).
__device__ __forceinline__ int swz(int j) { return swz_slot(j); }

struct TileGeo {
    int64_t sample;       // first sample of the tile
    int nsamples;         // valid samples in the tile (n < TB) else 1
    uint32_t fixed_val;   // global-bit values of the qubits outside the tile
    int64_t base;         // amplitude offset of local index 0
    int tile_in_sample;   // n >= TB: tile index within the sample
};

// The low bits of v deposited into the set bits of mask, lowest first.
__device__ __forceinline__ uint32_t deposit_bits(uint32_t v, uint32_t mask) {
    uint32_t r = 0;
    while (mask) {
        const uint32_t low = mask & (0u - mask);
        if (v & 1u) r |= low;
        v >>= 1;
        mask ^= low;
    }
    return r;
}

// Global bits of the qubits outside the tile, as a mask.
__device__ __forceinline__ uint32_t fixed_mask_of(const PassDesc& d) {
    uint32_t m = 0;
    for (int k = 0; k < d.nfixed; ++k) m |= 1u << d.fixed_gbit[k];
    return m;
}

// Geometry of tile t of a pass with tiles of 2^tile_bits amplitudes whose
// outside qubits are the global bits in fixed_mask (register arithmetic only).
__device__ __forceinline__ TileGeo tile_geo_m(int tile_bits, uint32_t fixed_mask, int64_t t, int n,
                                              int64_t batch) {
    TileGeo g;
    if (n >= tile_bits) {
        const int sh = n - tile_bits;  // tiles per sample = 2^sh
        g.sample = t >> sh;
        const uint32_t ti = (uint32_t)(t & ((int64_t(1) << sh) - 1));
        g.tile_in_sample = (int)ti;
        g.fixed_val = deposit_bits(ti, fixed_mask);
        g.base = (g.sample << n) + g.fixed_val;
        g.nsamples = 1;
    } else {
        int spt = 1 << (tile_bits - n);
        g.sample = t * spt;
        int64_t rem = batch - g.sample;
        g.nsamples = rem < spt ? (int)rem : spt;
        g.fixed_val = 0;
        g.base = g.sample << n;
        g.tile_in_sample = 0;
    }
    return g;
}

// global amplitude offset of the first element of run r
__device__ __forceinline__ int64_t run_offset(const PassDesc& d, int r) {
    int64_t off = 0;
    int hi = d.tile_bits - d.run_bits;
    for (int k = 0; k < hi; ++k)
        if ((r >> k) & 1) {
            int lb = d.run_bits + k;
            off += (lb < d.nq_tile) ? (int64_t(1) << d.gbit[lb]) : 0;
        }
    return off;
}

// float (probability) image of a tile: half the bytes of the state image
__device__ void issue_tile_store_f32(const PassDesc& d, const TileGeo& g, float* dstg, const float* src, int n,
                                     int lane) {
    if (n < d.tile_bits) {
        uint32_t bytes = (uint32_t)((int64_t)g.nsamples << n) * 4u;
        if (lane == 0) bulk_s2g(dstg + g.base, src, bytes);
        return;
    }
    int runs = 1 << (d.tile_bits - d.run_bits);
    uint32_t rb = (1u << d.run_bits) * 4u;
    for (int r = lane; r < runs; r += 32)
        bulk_s2g(dstg + g.base + run_offset(d, r), src + ((int64_t)r << d.run_bits), rb);
}

// ----------------------------------------------------- thread mapping --

struct ThreadMap {
    int regl[5];     // register bit k -> local bit (k < RB)
    int thr_off;     // local-index contribution of this thread's lane/warp bits
    uint32_t tglob;  // global-bit values of this thread's qubit thread bits | tile fixed bits
    int sample_off;  // sample offset within the tile (n < TB)
    // The swizzle is linear over GF(2) and the thread and register parts of a
    // local index have disjoint bits, so slot(r) = sw_base ^ XOR_k(bit k of r ? sw[k] : 0).
    int sw[5];
    int sw_base;
};

// Mapping encoding (OP_MAP y/z/w): y = RB register local bits (4 bits each),
// z = 5 lane local bits, w = warp local bits | (warp-bit count << 16).
template <int RB>
__device__ __forceinline__ void decode_map(const PassDesc& d, int32_t y, int32_t z, int32_t w, int tid,
                                           uint32_t fixed_val, ThreadMap& m) {
#pragma unroll
    for (int k = 0; k < RB; ++k) m.regl[k] = (y >> (4 * k)) & 15;
    int nw = (w >> 16) & 7;
    int off = 0, soff = 0;
    uint32_t tg = fixed_val;
    for (int k = 0; k < 5 + nw; ++k) {
        int lb = k < 5 ? ((z >> (4 * k)) & 15) : ((w >> (4 * (k - 5))) & 15);
        int bit = (tid >> k) & 1;
        off |= bit << lb;
        if (lb < d.nq_tile)
            tg |= (uint32_t)bit << d.gbit[lb];
        else
            soff |= bit << (lb - d.nq_tile);
    }
    m.thr_off = off;
    m.tglob = tg;
    m.sample_off = soff;
#pragma unroll
    for (int k = 0; k < RB; ++k) m.sw[k] = swz(1 << m.regl[k]);
    m.sw_base = swz(off);
}

template <int RB>
__device__ __forceinline__ int roff_rt(const ThreadMap& m, int r) {
    int o = 0;
#pragma unroll
    for (int k = 0; k < RB; ++k)
        if ((r >> k) & 1) o += 1 << m.regl[k];
    return o;
}

// Natural mapping: lanes = local bits 0..4 (32 consecutive amplitudes per
// warp access), registers = local bits 5..5+RB-1, warps = the bits above.
template <int RB>
__device__ __forceinline__ int nat_index(int r, int tid) {
    return (tid & 31) | (r << 5) | ((tid >> 5) << (5 + RB));
}

template <int TB, int RB>
struct NatMap {
    __host__ __device__ static constexpr int32_t regs() {
        int32_t v = 0;
        for (int k = 0; k < RB; ++k) v |= (5 + k) << (4 * k);
        return v;
    }
    __host__ __device__ static constexpr int32_t warps() {
        int32_t v = 0;
        for (int k = 0; k < TB - 5 - RB; ++k) v |= (5 + RB + k) << (4 * k);
        return v | ((TB - 5 - RB) << 16);
    }
    static constexpr int32_t y = regs();
    static constexpr int32_t z = 0x43210;
    static constexpr int32_t w = warps();
};

__device__ __forceinline__ bool loc_bit_thread(int32_t loc, uint32_t tglob) {
    return (tglob >> (loc & 31)) & 1;
}

__device__ __forceinline__ void load_slot(const RunArgs& A, const float4* smats, int32_t slot, int32_t flags,
                                          int64_t sample, float2 m[4]) {
    float4 u, v;
    if (!(flags & OPF_PER_SAMPLE) && slot < kSmemMats) {
        u = smats[2 * slot];
        v = smats[2 * slot + 1];
    } else {
        // lanes of a partial tile past the last sample compute on garbage that
        // is never stored; keep their table reads inside the table
        if (sample >= A.batch) sample = A.batch - 1;
        const float4* src = (flags & OPF_PER_SAMPLE)
                                ? reinterpret_cast<const float4*>(A.mats_ps + (sample * A.nslots_ps + slot) * 4)
                                : reinterpret_cast<const float4*>(A.mats + (int64_t)slot * 4);
        u = __ldg(src);
        v = __ldg(src + 1);
    }
    m[0] = make_float2(u.x, u.y);
    m[1] = make_float2(u.z, u.w);
    m[2] = make_float2(v.x, v.y);
    m[3] = make_float2(v.z, v.w);
}

// ------------------------------------------------ planar forward ops --

template <int RB>
__device__ __forceinline__ void pload_nat(PTile<RB>& t, const float2* buf, int tid) {
#pragma unroll
    for (int r = 0; r < (1 << RB); ++r) set_amp<RB>(t, r, buf[nat_index<RB>(r, tid)]);
}

// The tile in natural order into shared memory; physical register r holds
// logical amplitude r ^ xm.
template <int RB>
__device__ __forceinline__ void pstore_nat(const PTile<RB>& t, float2* buf, int tid, uint32_t xm) {
    const int x = (int)xm << 5;
#pragma unroll
    for (int r = 0; r < (1 << RB); ++r) buf[nat_index<RB>(r, tid) ^ x] = get_amp<RB>(t, r);
}

// The tile in natural order into shared memory from a mapping `em` (OP_MAP
// encoding) whose lanes are local bits 0..4; physical register r holds
// logical amplitude r ^ xm.  Register and warp bits are distinct local bits,
// so a register index's offset is the XOR of its bits' offsets.
template <int RB>
__device__ __forceinline__ void pstore_map(const PTile<RB>& t, float2* buf, const int32_t em[3], int tid,
                                           uint32_t xm) {
    int thr = tid & 31;
    const int nw = (em[2] >> 16) & 7;
    for (int k = 0; k < nw; ++k) thr |= ((tid >> (5 + k)) & 1) << ((em[2] >> (4 * k)) & 15);
    int ro[1 << RB];
    ro[0] = 0;
#pragma unroll
    for (int k = 0; k < RB; ++k) {
        const int bit = 1 << ((em[0] >> (4 * k)) & 15);
#pragma unroll
        for (int r = 0; r < (1 << k); ++r) ro[r + (1 << k)] = ro[r] | bit;
    }
    int xoff = 0;
#pragma unroll
    for (int k = 0; k < RB; ++k)
        if ((xm >> k) & 1) xoff ^= ro[1 << k];
#pragma unroll
    for (int r = 0; r < (1 << RB); ++r) buf[thr | (ro[r] ^ xoff)] = get_amp<RB>(t, r);
}

// Probabilities of the tile in natural order into shared memory; physical
// register r holds logical amplitude r ^ xm.
template <int RB>
__device__ __forceinline__ void pstore_probs(const PTile<RB>& t, float* pb, int tid, uint32_t xm) {
    const int x = (int)xm << 5;
#pragma unroll
    for (int k = 0; k < (1 << (RB - 1)); ++k) {
        const float2 p = vfma(t.I[k], t.I[k], vmul(t.R[k], t.R[k]));
        pb[nat_index<RB>(2 * k, tid) ^ x] = p.x;
        pb[nat_index<RB>(2 * k + 1, tid) ^ x] = p.y;
    }
}

// P0 partials of a tile that holds TB qubits of one sample (n >= TB), from
// the registers of the natural mapping (local bits 0..4 the lane, 5..4+RB the
// register index, the rest the warp; physical register r holds logical
// amplitude r ^ xm).  dst[b] = the sum of |amp|^2 over the tile's amplitudes
// whose local bit b is 0 (b < TB), dst[TB] = the tile's total.  Each thread
// sums its 2^RB probabilities per register bit value; each warp reduces its
// RB + 6 values (register-bit sums, the total, and the total of the lanes
// whose bit j is 0, j < 5) with a transposing butterfly (16 shuffles: lane L
// ends with the warp's sum of value L / 2); red[w][i] holds warp w's values,
// and threads 0..TB add them over the warps.  The caller synchronises the
// compute warps between the writes to red and the final sums.
template <int TB, int RB>
__device__ __forceinline__ void p0_warp_sums(const PTile<RB>& t, uint32_t xm, float (*red)[16], int tid, int lane) {
    constexpr int H = 1 << (RB - 1);
    float T[H];
    float z0 = 0.f, o0 = 0.f;
#pragma unroll
    for (int h = 0; h < H; ++h) {
        const float2 p = vfma(t.I[h], t.I[h], vmul(t.R[h], t.R[h]));  // registers 2h, 2h + 1
        T[h] = p.x + p.y;
        z0 += p.x;
        o0 += p.y;
    }
    float v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = 0.f;
    v[0] = (xm & 1u) ? o0 : z0;
#pragma unroll
    for (int k = 1; k < RB; ++k) {
        float z = 0.f, o = 0.f;
#pragma unroll
        for (int h = 0; h < H; ++h) {
            if ((h >> (k - 1)) & 1) o += T[h];
            else z += T[h];
        }
        v[k] = ((xm >> k) & 1u) ? o : z;
    }
    const float tot = z0 + o0;
    v[RB] = tot;
#pragma unroll
    for (int j = 0; j < 5; ++j) v[RB + 1 + j] = ((lane >> j) & 1) ? 0.f : tot;
    // transposing butterfly: after the step over lane bit b the lane keeps
    // the half of its values selected by that bit, summed with its partner's
#pragma unroll
    for (int w = 8; w >= 1; w >>= 1) {
        const int off = 2 * w;  // lane bits 4, 3, 2, 1
        const bool hi = (lane & off) != 0;
#pragma unroll
        for (int i = 0; i < w; ++i) {
            const float send = hi ? v[i] : v[i + w];
            const float keep = hi ? v[i + w] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
    if (!(lane & 1) && (lane >> 1) < RB + 6) red[tid >> 5][lane >> 1] = v[0];
}

template <int TB, int RB>
__device__ __forceinline__ void p0_tile_from_warps(const float (*red)[16], int tid, float* dst) {
    constexpr int NW = 1 << (TB - RB - 5);
    if (tid > TB) return;
    float acc = 0.f;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        float x;
        if (tid < 5) x = red[w][RB + 1 + tid];                  // lane bit
        else if (tid < 5 + RB) x = red[w][tid - 5];             // register bit
        else if (tid < TB) x = ((w >> (tid - 5 - RB)) & 1) ? 0.f : red[w][RB];  // warp bit
        else x = red[w][RB];                                    // total
        acc += x;
    }
    dst[tid] = acc;
}

// Exchange through planar shared memory (re plane, im plane), folding the
// pending X of the thread into the write addresses.
template <int RB, int K = 0>
__device__ __forceinline__ void pxwrite_k(float* plane, const PTile<RB>& t, const ThreadMap& m, int base, int amps) {
    const int slot = base ^ ((K & 1) ? m.sw[0] : 0) ^ ((K & 2) ? m.sw[1] : 0) ^ ((K & 4) ? m.sw[2] : 0) ^
                     ((K & 8) ? m.sw[3] : 0) ^ ((K & 16) ? m.sw[4] : 0);
    const float2 a = get_amp<RB>(t, K);
    plane[slot] = a.x;
    plane[slot + amps] = a.y;
    if constexpr (K + 1 < (1 << RB)) pxwrite_k<RB, K + 1>(plane, t, m, base, amps);
}
template <int RB, int K = 0>
__device__ __forceinline__ void pxread_k(const float* plane, PTile<RB>& t, const ThreadMap& m, int amps) {
    const int slot = m.sw_base ^ ((K & 1) ? m.sw[0] : 0) ^ ((K & 2) ? m.sw[1] : 0) ^ ((K & 4) ? m.sw[2] : 0) ^
                     ((K & 8) ? m.sw[3] : 0) ^ ((K & 16) ? m.sw[4] : 0);
    set_amp<RB>(t, K, make_float2(plane[slot], plane[slot + amps]));
    if constexpr (K + 1 < (1 << RB)) pxread_k<RB, K + 1>(plane, t, m, amps);
}

template <int RB>
__device__ __forceinline__ int xm_slot_offset(const ThreadMap& m, uint32_t xm) {
    int o = 0;
#pragma unroll
    for (int k = 0; k < RB; ++k)
        if ((xm >> k) & 1) o ^= m.sw[k];
    return o;
}

// One pass of one program over one state: an entry of a multi-job launch.
struct JobDesc {
    const PassDesc* pd;   // device pass descriptor
    const int4* ops;      // device ops of the pass
    RunArgs A;
    int32_t zero_init;    // start from |0..0> instead of loading the state
    int32_t pad;
    int64_t tiles;
};

template <int MAXJ>
struct JobTable {
    int32_t njobs;
    int32_t pad;
    int64_t begin[MAXJ + 1];  // first global tile of each job; begin[njobs] = total
    JobDesc job[MAXJ];
};

template <int MAXJ>
__device__ __forceinline__ int find_job(const JobTable<MAXJ>& jt, int64_t t) {
    int j = 0;
    while (j + 1 < jt.njobs && t >= jt.begin[j + 1]) ++j;
    return j;
}

// Exchange through the tile's buffer to the mapping (y, z, w) (OP_MAP
// encoding); the pending X of the thread is folded into the write addresses.
template <int TB, int RB>
__device__ __forceinline__ void exchange(PTile<RB>& pt, uint32_t& xm, ThreadMap& tm, float* plane,
                                         const PassDesc& d, int32_t y, int32_t z, int32_t w, int tid,
                                         uint32_t fixed_val) {
    cta_sync<(1 << (TB - RB))>();
    pxwrite_k<RB>(plane, pt, tm, tm.sw_base ^ xm_slot_offset<RB>(tm, xm), 1 << TB);
    xm = 0;
    cta_sync<(1 << (TB - RB))>();
    decode_map<RB>(d, y, z, w, tid, fixed_val, tm);
    pxread_k<RB>(plane, pt, tm, 1 << TB);
}

// ---------------------------------------------------- producer warps --

// The producer warps copy a tile as blocks of 2^cb amplitudes, cb being the
// number of low local bits that map to the same global bits: each block is
// contiguous in global memory and in the tile image, and moves with one bulk
// (TMA) copy.  Producer thread p takes blocks p, p + 32 P, ...; a block's
// global offset deposits its index into the tile's higher global bits.
struct BlockSide {
    int job = -1;         // job whose pass the side holds
    int cb;               // log2 amplitudes per block
    int nblk;             // blocks per tile (n >= TB)
    uint32_t fixed_mask;  // global bits of the qubits outside the tile
    int epi, ckpt;        // the pass's epilogue flags and checkpoint
    bool loads;           // the pass reads its tiles from the state
};

template <int TB, int MAXJ>
__device__ __forceinline__ void block_side(BlockSide& cs, const JobTable<MAXJ>& jt, int j) {
    if (cs.job == j) return;
    const PassDesc& pd = *jt.job[j].pd;
    int e = pd.run_bits;
    while (e < TB && pd.gbit[e] == e) ++e;
    cs.cb = e;
    cs.nblk = 1 << (TB - e);
    cs.fixed_mask = fixed_mask_of(pd);
    cs.epi = pd.epi;
    cs.ckpt = pd.ckpt;
    cs.loads = pd.init == INIT_LOAD && !jt.job[j].zero_init;
    cs.job = j;
}

// Global offset (amplitudes, within the tile) of block b.
template <int TB, int MAXJ>
__device__ __forceinline__ uint32_t block_offset(const JobTable<MAXJ>& jt, const BlockSide& cs, int b) {
    const PassDesc& pd = *jt.job[cs.job].pd;
    uint32_t o = 0;
    for (int k = 0; k < TB - cs.cb; ++k)
        if ((b >> k) & 1) o |= 1u << pd.gbit[cs.cb + k];
    return o;
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
                 : "memory");
}
template <int N>
__device__ __forceinline__ void producer_sync() {
    asm volatile("bar.sync 2, %0;" ::"n"(N) : "memory");
}
template <int N>
__device__ __forceinline__ bool producer_sync_and(bool v) {
    uint32_t r;
    asm volatile(
        "{ .reg .pred p, q; setp.ne.u32 p, %1, 0; bar.red.and.pred q, 2, %2, p; selp.u32 %0, 1, 0, q; }"
        : "=r"(r)
        : "r"((uint32_t)v), "n"(N)
        : "memory");
    return r != 0;
}

// The producer warps: for the CTA's i-th tile (buffer i % S) they first store
// tile i - S out of that buffer once the compute warps released it (empty
// barrier) and wait until the bulk copies have read it, then publish tile i's
// geometry, copy its per-sample matrices (Ops::stage) and load it into the
// buffer; the full barrier completes when every byte has landed.  Tiles whose
// pass does not load (|0..0> start, embedding) still get their geometry and
// matrices: the compute warps need them and the buffer.
template <int TB, int MAXJ, class Ops>
__device__ __forceinline__ void fwd_producer(const JobTable<MAXJ>& jt, float2* bufs, uint64_t* bar_full,
                                             uint64_t* bar_empty, TileGeo* s_geo, float4* staged, int ptid) {
    constexpr int AMPS = 1 << TB;
    constexpr int S = fwd_stages(TB);
    constexpr int PT = 32 * fwd_producer_warps(TB);
    const int lane = ptid & 31;
    const int64_t total = jt.begin[jt.njobs];
    const int64_t G = gridDim.x;
    const int64_t t0 = blockIdx.x;
    const int64_t mine = (total - t0 + G - 1) / G;  // tiles of this CTA
    BlockSide ld, st;
    // offsets of this thread's blocks ptid + PT k of each side (tiles of at
    // most KB PT blocks; more, smaller blocks are located on the fly)
    constexpr int KB = ((1 << (TB - 6)) + PT - 1) / PT;
    uint32_t st_off[KB], ld_off[KB];
    int failed_job = -1;
    int64_t failed_tile = -1;
    for (int64_t i = 0; i < mine + S; ++i) {
        const int s = (int)(i % S);
        float2* buf = bufs + s * AMPS;
        if (i >= S) {
            const int64_t t = t0 + (i - S) * G;
            const int j = find_job(jt, t);
            const bool released = mbar_wait(bar_empty + s, (uint32_t)((i / S - 1) & 1));
            if (!producer_sync_and<PT>(released)) {
                failed_job = j;
                failed_tile = t;
                break;
            }
            if (st.job != j) {
                block_side<TB>(st, jt, j);
#pragma unroll
                for (int k = 0; k < KB; ++k)
                    st_off[k] = ptid + PT * k < st.nblk ? block_offset<TB>(jt, st, ptid + PT * k) : 0;
            }
            if (st.epi & EPI_STORE) {
                const RunArgs& A = jt.job[j].A;
                const TileGeo g = tile_geo_m(TB, st.fixed_mask, t - jt.begin[j], A.n, A.batch);
                float2* ck = st.ckpt >= 0 ? A.ckpt + (int64_t)st.ckpt * (A.batch << A.n) : nullptr;
                if (A.n < TB) {  // whole samples: one contiguous image
                    if (ptid == 0) {
                        const uint32_t bytes = (uint32_t)(((int64_t)g.nsamples << A.n) * 8);
                        bulk_s2g(A.state + g.base, buf, bytes);
                        if (ck) bulk_s2g(ck + g.base, buf, bytes);
                    }
                } else {
                    const uint32_t bytes = 8u << st.cb;
                    for (int b = ptid, k = 0; b < st.nblk; b += PT, ++k) {
                        const uint32_t off = k < KB ? st_off[k < KB ? k : 0] : block_offset<TB>(jt, st, b);
                        bulk_s2g(A.state + g.base + off, buf + ((int64_t)b << st.cb), bytes);
                        if (ck) bulk_s2g(ck + g.base + off, buf + ((int64_t)b << st.cb), bytes);
                    }
                }
                bulk_commit();
                bulk_wait_read0();  // this thread's copies have read the buffer
            }
            producer_sync<PT>();  // every copy out of the buffer has read it
        }
        if (i < mine) {
            const int64_t t = t0 + i * G;
            const int j = find_job(jt, t);
            if (ld.job != j) {
                block_side<TB>(ld, jt, j);
#pragma unroll
                for (int k = 0; k < KB; ++k)
                    ld_off[k] = ptid + PT * k < ld.nblk ? block_offset<TB>(jt, ld, ptid + PT * k) : 0;
            }
            const RunArgs& A = jt.job[j].A;
            const TileGeo g = tile_geo_m(TB, ld.fixed_mask, t - jt.begin[j], A.n, A.batch);
            if (ptid == 0) s_geo[s] = g;  // published by this thread's arrive below
            uint32_t mine_bytes = 0;
            if (ld.loads) {
                if (A.n < TB) {
                    if (ptid == 0) mine_bytes = (uint32_t)(((int64_t)g.nsamples << A.n) * 8);
                } else {
                    for (int b = ptid; b < ld.nblk; b += PT) mine_bytes += 8u << ld.cb;
                }
            }
            uint32_t warp_bytes = __reduce_add_sync(0xffffffffu, mine_bytes);
            if (ptid < 32) warp_bytes += Ops::kStagedBytes;
            if (lane == 0) mbar_arrive_expect_tx(bar_full + s, warp_bytes);
            __syncwarp();
            if (ptid < 32) Ops::stage(A, g, staged + s * (2 * kStagedPerSlot), bar_full + s, lane);
            if (ld.loads) {
                if (A.n < TB) {
                    if (ptid == 0) bulk_g2s(buf, A.state + g.base, mine_bytes, bar_full + s);
                } else {
                    const uint32_t bytes = 8u << ld.cb;
                    for (int b = ptid, k = 0; b < ld.nblk; b += PT, ++k) {
                        const uint32_t off = k < KB ? ld_off[k < KB ? k : 0] : block_offset<TB>(jt, ld, b);
                        bulk_g2s(buf + ((int64_t)b << ld.cb), A.state + g.base + off, bytes, bar_full + s);
                    }
                }
            }
        }
    }
    bulk_wait_all0();  // this thread's stores have completed before it leaves
    if (failed_job >= 0 && ptid == 0) report_timeout(jt.job[failed_job].A.status, kSiteFwdProducer, failed_tile);
}

// Body of the forward pass kernel.  One persistent CTA per SM walks the tiles
// of every job of the launch (the passes of independent programs / states,
// e.g. several serving requests of different widths); a single-program
// forward is a one-job launch.  The CTA's last warps are producers
// (fwd_producer): they move tiles between global memory and a ring of three
// shared-memory buffers, so the compute warps only read a tile out of its
// buffer into registers, run the pass's gate program on it (Ops::apply,
// exchanging through the same buffer), and write the result back.
template <int TB, int RB, int MAXJ, class Ops>
__device__ __forceinline__ void fwd_pass_body(const JobTable<MAXJ>& jt) {
    constexpr int NT = 1 << (TB - RB);
    constexpr int AMPS = 1 << TB;
    constexpr int S = fwd_stages(TB);
    static_assert(S == 3, "the producer ring is three tile buffers");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float2* bufs = reinterpret_cast<float2*>(smem_raw);
    int4* s_ops = reinterpret_cast<int4*>(bufs + S * AMPS);         // [kSmemOps]
    float4* s_mats = reinterpret_cast<float4*>(s_ops + kSmemOps);   // [kSmemMats][2]
    uint64_t* bar_full = reinterpret_cast<uint64_t*>(s_mats + 2 * kSmemMats);  // [S]
    uint64_t* bar_empty = bar_full + S;                                        // [S]
    __shared__ PassDesc sd;
    __shared__ RunArgs sa;
    __shared__ TileGeo s_geo[S];  // geometry of the tile in each buffer (written by the producer)
    // per-warp P0 sums of the register epilogue, by tile parity (every tile
    // passes a compute-warp barrier after warp 0 read the previous parity)
    __shared__ float s_red[2][1 << (TB - RB - 5)][16];

    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(bar_full + s, fwd_producer_warps(TB));  // lane 0 of every producer warp
            mbar_init(bar_empty + s, NT / 32);  // lane 0 of every compute warp
        }
    }
    __syncthreads();  // the only barrier the producer joins
    if (tid >= NT) {
        fwd_producer<TB, MAXJ, Ops>(jt, bufs, bar_full, bar_empty, s_geo, reinterpret_cast<float4*>(s_ops),
                                    tid - NT);
        return;
    }

    const int lane = tid & 31;
    const int64_t total = jt.begin[jt.njobs];
    const int64_t G = gridDim.x;
    const int64_t t0 = blockIdx.x;
    int cur_job = -1;
    int iter = 0;
    bool ok = true;
    int64_t failed_tile = -1;
    for (int64_t t = t0; t < total; t += G, ++iter) {
        const int slot = iter % S;
        float2* buf = bufs + slot * AMPS;
        const int j = find_job(jt, t);
        if (j != cur_job) {
            cta_sync<NT>();  // nobody reads the previous job's descriptors any more
            if (tid == 0) {
                sd = *jt.job[j].pd;
                sa = jt.job[j].A;
            }
            // the pass's op list (when Ops reads it) and the shared matrix
            // table, staged once per job
            if (Ops::kStageOps) {
                const int4* gops = jt.job[j].ops;
                const int nops = jt.job[j].pd->op_count;
                for (int i = tid; i < nops && i < kSmemOps; i += NT) s_ops[i] = __ldg(gops + i);
            }
            const int nm = jt.job[j].A.nslots_shared < kSmemMats ? jt.job[j].A.nslots_shared : kSmemMats;
            const float4* gm = reinterpret_cast<const float4*>(jt.job[j].A.mats);
            for (int i = tid; i < 2 * nm; i += NT) s_mats[i] = __ldg(gm + i);
            cta_sync<NT>();
            cur_job = j;
        }
        const PassDesc& d = sd;
        const RunArgs& A = sa;
        const int4* ops = jt.job[j].ops;
        const int n = A.n;
        // a compiled pass knows its init and epilogue kinds (Ops::kInit / kEpi
        // >= 0): the code of the other kinds is not compiled into it
        const int init = Ops::kInit >= 0 ? Ops::kInit : d.init;
        const int epi = Ops::kEpi >= 0 ? Ops::kEpi : d.epi;
        const bool load_in = init == INIT_LOAD && !jt.job[j].zero_init;
        // the tile's per-sample matrices (compiled passes) in the buffer's
        // share of the op-list area
        const float4* const staged = reinterpret_cast<const float4*>(s_ops) + slot * (2 * kStagedPerSlot);
        const bool landed = mbar_wait(bar_full + slot, (uint32_t)((iter / S) & 1));
        if (!cta_sync_and<NT>(landed)) {
            ok = false;
            failed_tile = t;
            break;
        }
        const TileGeo g = s_geo[slot];
        PTile<RB> pt;
        uint32_t xm = 0;  // pending thread-controlled X per register bit
        ThreadMap tm;
        if (load_in) {
            pload_nat<RB>(pt, buf, tid);
            decode_map<RB>(d, NatMap<TB, RB>::y, NatMap<TB, RB>::z, NatMap<TB, RB>::w, tid, g.fixed_val, tm);
        } else {
            if (init == INIT_EMBED)
                decode_map<RB>(d, d.init_map[0], d.init_map[1], d.init_map[2], tid, g.fixed_val, tm);
            else
                decode_map<RB>(d, NatMap<TB, RB>::y, NatMap<TB, RB>::z, NatMap<TB, RB>::w, tid, g.fixed_val, tm);
            int64_t smp = g.sample + tm.sample_off;
            if (init == INIT_EMBED && smp < A.batch) {
                // amplitude = prod over qubits of the per-sample factor of its bit
                const float2* fac = A.embfac + smp * n * 2;
                float2 c = make_float2(1.f, 0.f);
                uint32_t regmask = 0;
                for (int k = 0; k < RB; ++k) regmask |= 1u << d.gbit[tm.regl[k]];
                // (a loop unrolled to 32 bits, to issue every factor's load
                // ahead of the products, measured slower)
                for (int b = 0; b < n; ++b) {
                    if (regmask & (1u << b)) continue;
                    c = cmul(c, fac[2 * (n - 1 - b) + ((tm.tglob >> b) & 1)]);
                }
                float2 a[1 << RB];
                a[0] = c;
#pragma unroll
                for (int k = 0; k < RB; ++k) {
                    int b = d.gbit[tm.regl[k]];
                    float2 f0 = fac[2 * (n - 1 - b)], f1 = fac[2 * (n - 1 - b) + 1];
#pragma unroll
                    for (int r = 0; r < (1 << k); ++r) {
                        a[r + (1 << k)] = cmul(a[r], f1);
                        a[r] = cmul(a[r], f0);
                    }
                }
#pragma unroll
                for (int r = 0; r < (1 << RB); ++r) set_amp<RB>(pt, r, a[r]);
            } else if (init == INIT_EMBED) {
#pragma unroll
                for (int r = 0; r < (1 << RB); ++r) set_amp<RB>(pt, r, make_float2(0.f, 0.f));
            } else {
                // |0..0>: amplitude 1 where every qubit bit (in and outside the tile) is 0
                const int qmask = (1 << d.nq_tile) - 1;
#pragma unroll
                for (int r = 0; r < (1 << RB); ++r) {
                    bool origin = g.fixed_val == 0 && ((tm.thr_off + roff_rt<RB>(tm, r)) & qmask) == 0;
                    set_amp<RB>(pt, r, make_float2(origin ? 1.f : 0.f, 0.f));
                }
            }
        }
        // ---- the gate program of this pass ----
        // (the op list when Ops reads it, else the tile's staged matrices)
        Ops::template apply<TB, RB>(pt, xm, tm, d, A, ops,
                                    Ops::kStageOps ? s_ops : reinterpret_cast<const int4*>(staged), s_mats,
                                    reinterpret_cast<float*>(buf), g.sample, g.fixed_val, tid);
        // ---- epilogue (the planner left the natural mapping, or for a pass
        // that only stores, a mapping with natural lanes: d.end_map) ----
        const int64_t smp0 = g.sample;
        if ((epi & EPI_P0) && !(epi & EPI_PROBS) && d.nq_tile == TB) {
            // one sample per tile: sums from the registers, no pass through `buf`
            float(*red)[16] = s_red[iter & 1];
            p0_warp_sums<TB, RB>(pt, xm, red, tid, lane);
            cta_sync<NT>();
            p0_tile_from_warps<TB, RB>(
                red, tid, A.p0part + ((smp0 * (int64_t(1) << (n - TB)) + g.tile_in_sample) * (TB + 1)));
        } else if (epi & (EPI_PROBS | EPI_P0)) {
            cta_sync<NT>();  // all exchange reads of `buf` are done
            float* pb = reinterpret_cast<float*>(buf);
            pstore_probs<RB>(pt, pb, tid, xm);
            if (epi & EPI_PROBS) {
                fence_proxy_async();
                cta_sync<NT>();
                if (tid < 32) {
                    issue_tile_store_f32(d, g, A.out, pb, n, lane);
                    bulk_commit();
                    bulk_wait_read0();
                }
            }
            cta_sync<NT>();
            if (epi & EPI_P0) {
                // phase A: thread t owns the 2^RB consecutive probabilities of chunk t
                constexpr int CH = 1 << RB;
                float* ptot = pb + AMPS;          // [NT]
                float* psub = ptot + NT;          // [RB][NT]
                const float* chunk = pb + tid * CH;
                float tot = 0.f, sj[RB];
#pragma unroll
                for (int jj = 0; jj < RB; ++jj) sj[jj] = 0.f;
#pragma unroll
                for (int k = 0; k < CH; ++k) {
                    int idx = (k + tid) & (CH - 1);  // rotated start spreads the banks
                    float v = chunk[idx];
                    tot += v;
#pragma unroll
                    for (int jj = 0; jj < RB; ++jj) sj[jj] += ((idx >> jj) & 1) ? 0.f : v;
                }
                ptot[tid] = tot;
#pragma unroll
                for (int jj = 0; jj < RB; ++jj) psub[jj * NT + tid] = sj[jj];
                cta_sync<NT>();
                // phase B: (sample, local bit) items
                const int nq = d.nq_tile;
                const int cps = 1 << (nq - RB);           // chunks (threads) per sample
                const int spt = NT / cps;                 // samples per tile
                const int items = spt * (nq + 1);
                const int64_t tps = (n >= TB) ? (int64_t(1) << (n - TB)) : 1;
                if (cps >= 32) {
                    const int warp = tid >> 5;
                    for (int it = warp; it < items; it += NT / 32) {
                        int s = it / (nq + 1), jj = it % (nq + 1);
                        float acc = 0.f;
                        for (int c = lane; c < cps; c += 32) {
                            int t2 = s * cps + c;
                            if (jj < RB) acc += psub[jj * NT + t2];
                            else if (jj < nq) acc += ((t2 >> (jj - RB)) & 1) ? 0.f : ptot[t2];
                            else acc += ptot[t2];
                        }
                        for (int o2 = 16; o2 > 0; o2 >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o2);
                        if (lane == 0 && s < g.nsamples) {
                            int64_t smp = smp0 + s;
                            float* dst = A.p0part + ((smp * tps + g.tile_in_sample) * (TB + 1));
                            dst[jj < nq ? jj : TB] = acc;
                        }
                    }
                } else {
                    for (int it = tid; it < items; it += NT) {
                        int s = it / (nq + 1), jj = it % (nq + 1);
                        float acc = 0.f;
                        for (int c = 0; c < cps; ++c) {
                            int t2 = s * cps + c;
                            if (jj < RB) acc += psub[jj * NT + t2];
                            else if (jj < nq) acc += ((t2 >> (jj - RB)) & 1) ? 0.f : ptot[t2];
                            else acc += ptot[t2];
                        }
                        if (s < g.nsamples) {
                            int64_t smp = smp0 + s;
                            float* dst = A.p0part + ((smp * tps + g.tile_in_sample) * (TB + 1));
                            dst[jj < nq ? jj : TB] = acc;
                        }
                    }
                }
            }
        }
        if (epi & EPI_STORE) {
            cta_sync<NT>();  // all reads of `buf` (exchanges, probabilities) are done
            const bool nat_end = Ops::kEndNatural >= 0
                                     ? Ops::kEndNatural == 1
                                     : (d.end_map[0] == NatMap<TB, RB>::y && d.end_map[2] == NatMap<TB, RB>::w);
            if (nat_end)
                pstore_nat<RB>(pt, buf, tid, xm);
            else
                pstore_map<RB>(pt, buf, d.end_map, tid, xm);
            fence_proxy_async();  // the bulk copies that store the buffer see these writes
        }
        // the warp is done with the buffer (and its part of the state image
        // is in it when the pass stores): the producer writes it out and
        // refills the buffer
        __syncwarp();
        if (lane == 0) mbar_arrive(bar_empty + slot);
    }
    if (!ok && tid == 0) report_timeout(sa.status, kSiteFwdCompute, failed_tile);
    if (tid < 32) bulk_wait_all0();  // probability stores have completed
}


}  // namespace qg

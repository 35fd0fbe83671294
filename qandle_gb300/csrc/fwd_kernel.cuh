// Forward pass kernel shared by the prebuilt op interpreter (fused.cu) and
// by the pass kernels the library compiles at run time with NVRTC for one
// program (jit.cpp).  Everything here is device code that needs no host
// header, so the same text is handed to NVRTC.
//
// A pass walks tiles of 2^TB amplitudes: each tile is loaded by per-thread
// async copies (cp.async) into one of a ring of shared-memory buffers, so
// later tiles stream in while the current one is computed, and stored
// straight from registers.  A thread holds 2^RB amplitudes in registers (planar.cuh); the
// gate program of the pass runs on them (`Ops`), exchanging through the
// tile's buffer when the register qubits change; the epilogue stores the
// tile, its probabilities or P0 partials.
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
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void bulk_wait_all0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ------------------------------------------------------- tile geometry --

// Swizzled shared-memory slot of local index j: the low 5 bits are XORed with
// the 5-bit groups above them, so 32 lanes whose local bits have distinct
// (bit mod 5) hit the 32 distinct 4-byte banks of a planar exchange.
__device__ __forceinline__ int swz(int j) { return j ^ (((j >> 5) ^ (j >> 10)) & 31); }

struct TileGeo {
    int64_t sample;       // first sample of the tile
    int nsamples;         // valid samples in the tile (n < TB) else 1
    uint32_t fixed_val;   // global-bit values of the qubits outside the tile
    int64_t base;         // amplitude offset of local index 0
    int tile_in_sample;   // n >= TB: tile index within the sample
};

__device__ __forceinline__ TileGeo tile_geo(const PassDesc& d, int64_t t, int n, int64_t batch) {
    TileGeo g;
    if (n >= d.tile_bits) {
        int64_t tps = int64_t(1) << (n - d.tile_bits);
        g.sample = t / tps;
        int64_t ti = t - g.sample * tps;
        g.tile_in_sample = (int)ti;
        uint32_t fv = 0;
        for (int k = 0; k < d.nfixed; ++k) fv |= (uint32_t)((ti >> k) & 1) << d.fixed_gbit[k];
        g.fixed_val = fv;
        g.base = (g.sample << n) + fv;
        g.nsamples = 1;
    } else {
        int spt = 1 << (d.tile_bits - n);
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

// Per-thread async copies (cp.async, 16 bytes = 2 amplitudes each) of one
// tile's state image into dst in local-index order.  Every thread of the CTA
// issues 2^(RB-1) copies; thread tid copies chunks tid, tid + NT, ..., so a
// warp covers 512 contiguous bytes of a run.  Unlike one engine working
// through a tile's runs (bulk copies), the load/store units of all warps keep
// many small copies in flight, which scattered 512-byte runs need.  Local
// bit 0 is global bit 0 (runs are at least 2 amplitudes), so a chunk is
// contiguous; higher local bits add their global strides.  The caller
// commits the copies as one group.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <int TB, int RB>
__device__ __forceinline__ void thread_tile_load(const PassDesc& d, const TileGeo& g, const float2* src,
                                                 float2* dst, int n, int tid) {
    constexpr int NT = 1 << (TB - RB);
    constexpr int PER = 1 << (RB - 1);  // chunks per thread
    const float2* base = src + g.base;
    if (n < TB) {  // whole samples: the tile image is contiguous
        const int lim = (int)(((int64_t)g.nsamples << n) >> 1);
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            const int c = tid + i * NT;
            if (c < lim) cp_async16(dst + 2 * c, base + 2 * c);
        }
        return;
    }
    uint32_t thr = 0;
#pragma unroll
    for (int k = 0; k < TB - RB; ++k) thr |= (uint32_t)((tid >> k) & 1) << d.gbit[1 + k];
    uint32_t st[RB - 1];
#pragma unroll
    for (int k = 0; k < RB - 1; ++k) st[k] = 1u << d.gbit[TB - RB + 1 + k];
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        uint32_t off = thr;
#pragma unroll
        for (int k = 0; k < RB - 1; ++k)
            if ((i >> k) & 1) off ^= st[k];
        cp_async16(dst + 2 * (tid + i * NT), base + off);
    }
}

// Tiles of at most 2^this contiguous blocks are stored by bulk copies.
constexpr int kMaxBulkStoreBlocksLog2 = 4;

// Local bits below the returned count map to the same global bits, so the
// tile image is made of contiguous blocks of 2^count amplitudes (at least
// the runs).
__device__ __forceinline__ int contiguous_bits(const PassDesc& d) {
    int e = d.run_bits;
    while (e < d.tile_bits && d.gbit[e] == e) ++e;
    return e;
}

// Bulk copies of a tile's state image from shared memory (local-index order)
// to global memory, one per contiguous block; issued by the 32 lanes of one
// warp, which then commit them as their bulk group.
__device__ void issue_tile_store(const PassDesc& d, const TileGeo& g, float2* dstg, const float2* src, int n,
                                 int lane) {
    if (n < d.tile_bits) {
        const uint32_t bytes = (uint32_t)((int64_t)g.nsamples << n) * 8u;
        if (lane == 0) bulk_s2g(dstg + g.base, src, bytes);
        return;
    }
    const int e = contiguous_bits(d);
    const int blocks = 1 << (d.tile_bits - e);
    const uint32_t bytes = (1u << e) * 8u;
    for (int r = lane; r < blocks; r += 32) {
        int64_t off = 0;
        for (int k = 0; k < d.tile_bits - e; ++k)
            if ((r >> k) & 1) off += int64_t(1) << d.gbit[e + k];
        bulk_s2g(dstg + g.base + off, src + ((int64_t)r << e), bytes);
    }
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

// Store a tile in the natural mapping straight from registers to global
// memory.  The lanes hold 32 consecutive amplitudes of a run, so a warp
// store covers 256 contiguous bytes whenever the lanes share their pending
// X; no shared-memory staging, so the tile's buffer is free at once.
// Physical register r holds logical amplitude r ^ xm.  Local bits map to
// distinct global bits, so offsets of the register part combine by XOR.
template <int RB>
__device__ __forceinline__ void pstore_global(const PTile<RB>& t, uint32_t xm, const PassDesc& d,
                                              const TileGeo& g, float2* dst, int n, int tid) {
    float2* base = dst + g.base;
    if (n < d.tile_bits) {  // whole samples: the tile image is contiguous
        const int64_t lim = (int64_t)g.nsamples << n;
#pragma unroll
        for (int r = 0; r < (1 << RB); ++r) {
            const int j = nat_index<RB>(r ^ (int)xm, tid);
            if (j < lim) base[j] = get_amp<RB>(t, r);
        }
        return;
    }
    uint32_t rs[RB];
#pragma unroll
    for (int k = 0; k < RB; ++k) rs[k] = 1u << d.gbit[5 + k];
    uint32_t c = 0;
#pragma unroll
    for (int k = 0; k < 5; ++k) c |= (uint32_t)((tid >> k) & 1) << d.gbit[k];
    for (int k = 0; k < d.tile_bits - 5 - RB; ++k) c |= (uint32_t)((tid >> (5 + k)) & 1) << d.gbit[5 + RB + k];
#pragma unroll
    for (int k = 0; k < RB; ++k) c ^= ((xm >> k) & 1u) ? rs[k] : 0u;
    uint32_t off[1 << RB];
    off[0] = c;
#pragma unroll
    for (int k = 0; k < RB; ++k)
#pragma unroll
        for (int r = 0; r < (1 << k); ++r) off[r + (1 << k)] = off[r] ^ rs[k];
#pragma unroll
    for (int r = 0; r < (1 << RB); ++r) base[off[r]] = get_amp<RB>(t, r);
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
    __syncthreads();
    pxwrite_k<RB>(plane, pt, tm, tm.sw_base ^ xm_slot_offset<RB>(tm, xm), 1 << TB);
    xm = 0;
    __syncthreads();
    decode_map<RB>(d, y, z, w, tid, fixed_val, tm);
    pxread_k<RB>(plane, pt, tm, 1 << TB);
}

// Body of the forward pass kernel.  One persistent CTA per SM walks the tiles
// of every job of the launch (the passes of independent programs / states,
// e.g. several serving requests of different widths); a single-program
// forward is a one-job launch.  Ops::apply runs the pass's gate program on
// the thread's tile.
template <int TB, int RB, int MAXJ, class Ops>
__device__ __forceinline__ void fwd_pass_body(const JobTable<MAXJ>& jt) {
    constexpr int NT = 1 << (TB - RB);
    constexpr int AMPS = 1 << TB;
    constexpr int S = fwd_stages(TB);  // tile buffers: loads run S-1 tiles ahead
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float2* bufs = reinterpret_cast<float2*>(smem_raw);
    int4* s_ops = reinterpret_cast<int4*>(bufs + S * AMPS);         // [kSmemOps]
    float4* s_mats = reinterpret_cast<float4*>(s_ops + kSmemOps);   // [kSmemMats][2]
    __shared__ PassDesc sd;
    __shared__ RunArgs sa;

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int64_t total = jt.begin[jt.njobs];

    auto tile_loads = [&](int j) -> bool {
        return jt.job[j].pd->init == INIT_LOAD && !jt.job[j].zero_init;
    };
    // Buffer ring (S = 3): tile t computes in buffer t % 3 while tile t + 1
    // loads into the next buffer and the bulk store of tile t - 1 reads out of
    // the previous one.  Every thread commits exactly one copy group per
    // prefetch (empty when there is nothing to load), so "tile t has landed"
    // is cp.async.wait_group 0 followed by a CTA barrier; warp 0 commits one
    // bulk-store group per tile (empty when the tile stores nothing).
    auto issue_prefetch = [&](int64_t t, float2* dst) {
        if (t < total) {
            const int j = find_job(jt, t);
            if (tile_loads(j)) {
                const PassDesc& pd = *jt.job[j].pd;
                const RunArgs& ra = jt.job[j].A;
                TileGeo gn = tile_geo(pd, t - jt.begin[j], ra.n, ra.batch);
                thread_tile_load<TB, RB>(pd, gn, ra.state, dst, ra.n, tid);
            }
        }
        cp_async_commit();
    };

    static_assert(S == 3, "the store write-behind needs three tile buffers");
    const int64_t t0 = blockIdx.x;
    issue_prefetch(t0, bufs);
    int cur_job = -1;
    int iter = 0;
    for (int64_t t = t0; t < total; t += gridDim.x, ++iter) {
        const int slot = iter % S;
        float2* buf = bufs + slot * AMPS;
        const int j = find_job(jt, t);
        if (j != cur_job) {
            __syncthreads();  // nobody reads the previous job's descriptors any more
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
            __syncthreads();
            cur_job = j;
        }
        const PassDesc& d = sd;
        const RunArgs& A = sa;
        const int4* ops = jt.job[j].ops;
        const int n = A.n;
        const bool load_in = tile_loads(j);
        TileGeo g = tile_geo(d, t - jt.begin[j], n, A.batch);
        PTile<RB> pt;
        uint32_t xm = 0;  // pending thread-controlled X per register bit
        ThreadMap tm;
        // per-tile data of Ops (in the op-list area when it is not staged;
        // two halves alternate by tile), published by the barrier below
        Ops::template tile_start<TB, RB>(A, g, reinterpret_cast<float4*>(s_ops) + (iter & 1) * (kSmemOps / 2),
                                         tid);
        cp_async_wait<0>();  // this thread's copies of tile t have landed
        // warp 0: the bulk store of tile t - 2 has read its buffer out (it had
        // all of tile t - 1 to do so), so that buffer can take tile t + 1
        if (tid < 32) bulk_wait_read<1>();
        __syncthreads();  // tile t has landed everywhere; buffer (t + 1) % 3 is free
        if (load_in) {
            pload_nat<RB>(pt, buf, tid);
            decode_map<RB>(d, NatMap<TB, RB>::y, NatMap<TB, RB>::z, NatMap<TB, RB>::w, tid, g.fixed_val, tm);
        } else {
            if (d.init == INIT_EMBED)
                decode_map<RB>(d, d.init_map[0], d.init_map[1], d.init_map[2], tid, g.fixed_val, tm);
            else
                decode_map<RB>(d, NatMap<TB, RB>::y, NatMap<TB, RB>::z, NatMap<TB, RB>::w, tid, g.fixed_val, tm);
            int64_t smp = g.sample + tm.sample_off;
            if (d.init == INIT_EMBED && smp < A.batch) {
                // amplitude = prod over qubits of the per-sample factor of its bit
                const float2* fac = A.embfac + smp * n * 2;
                float2 c = make_float2(1.f, 0.f);
                uint32_t regmask = 0;
                for (int k = 0; k < RB; ++k) regmask |= 1u << d.gbit[tm.regl[k]];
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
            } else if (d.init == INIT_EMBED) {
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
        // prefetch tile t + 1 into the buffer tile t - 2 used
        issue_prefetch(t + (int64_t)gridDim.x, bufs + ((iter + 1) % S) * AMPS);
        // ---- the gate program of this pass ----
        // (the op list when Ops reads it, else this tile's half of the staged data)
        Ops::template apply<TB, RB>(pt, xm, tm, d, A, ops,
                                    Ops::kStageOps ? s_ops : s_ops + (iter & 1) * (kSmemOps / 2), s_mats,
                                    reinterpret_cast<float*>(buf), g.sample, g.fixed_val, tid);
        // ---- epilogue (the planner left the natural mapping) ----
        const bool bulk_store = n < TB || d.tile_bits - contiguous_bits(d) <= kMaxBulkStoreBlocksLog2;
        const bool epi_uses_buf = (d.epi & (EPI_PROBS | EPI_P0)) || ((d.epi & EPI_STORE) && bulk_store);
        if (epi_uses_buf) __syncthreads();  // all exchange reads of `buf` are done
        const int64_t smp0 = g.sample;
        // A tile made of a few large contiguous blocks is written back by bulk
        // copies that read the buffer while the next tile computes; a tile of
        // many small runs is stored straight from registers (one copy engine
        // working through many 512-byte runs is slower than the warps).
        if (d.epi & EPI_STORE) {
            if (bulk_store) {
                pstore_nat<RB>(pt, buf, tid, xm);
                fence_proxy_async();
                __syncthreads();
                if (tid < 32) {
                    issue_tile_store(d, g, A.state, buf, n, lane);
                    if (d.ckpt >= 0)
                        issue_tile_store(d, g, A.ckpt + (int64_t)d.ckpt * (A.batch << n), buf, n, lane);
                }
            } else {
                pstore_global<RB>(pt, xm, d, g, A.state, n, tid);
                if (d.ckpt >= 0)
                    pstore_global<RB>(pt, xm, d, g, A.ckpt + (int64_t)d.ckpt * (A.batch << n), n, tid);
            }
        }
        if (d.epi & (EPI_PROBS | EPI_P0)) {
            if ((d.epi & EPI_STORE) && bulk_store) {  // the probabilities reuse the buffer: let the store read it first
                if (tid < 32) {
                    bulk_commit();
                    bulk_wait_read0();
                }
                __syncthreads();
            }
            float* pb = reinterpret_cast<float*>(buf);
            pstore_probs<RB>(pt, pb, tid, xm);
            if (d.epi & EPI_PROBS) {
                fence_proxy_async();
                __syncthreads();
                if (tid < 32) {
                    issue_tile_store_f32(d, g, A.out, pb, n, lane);
                    bulk_commit();
                    bulk_wait_read0();
                }
            }
            __syncthreads();
            if (d.epi & EPI_P0) {
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
                __syncthreads();
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
        if (tid < 32) bulk_commit();  // this tile's store group (possibly empty)
        // No barrier here: the next tile's first barrier orders everything
        // that touches shared memory (the staged per-sample data alternates
        // between two halves, and `buf` is refilled only two tiles later).
    }
    if (tid < 32) bulk_wait_all0();
}


}  // namespace qg

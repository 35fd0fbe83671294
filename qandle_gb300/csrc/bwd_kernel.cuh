// Backward (adjoint) pass kernel shared by the prebuilt op interpreter
// (fused.cu) and the backward pass kernels compiled at run time (jit.cpp).
// Device code only, handed to NVRTC as text.
//
// A backward pass walks tiles of psi (the state) and lambda (the cotangent):
// a producer warp moves both between global memory and two shared-memory
// slots with bulk copies, the pass's inverse gates act on both in registers
// with one shared pending-X mask, and every rotation first leaves its
// gradient partial Im<lambda|P|psi> in shared memory; the partials of a tile
// are reduced per sample in a fixed order.
#pragma once
#include "fwd_kernel.cuh"

namespace qg {

// Gradient partial of a rotation with generator axis on register bit P, with
// the pending X folded in: the physical pair order turns the generator G into
// X G X (= -G for Y and Z).
template <int P, int RB>
__device__ __forceinline__ float pgrad_at(const PTile<RB>& ps, const PTile<RB>& ls, int axis, uint32_t xm) {
    const float g = pgrad<P, RB>(ps, ls, axis);
    return (((xm >> P) & 1u) && axis != AX_X) ? -g : g;
}

// Record a thread's gradient partial for grad slot `rel` of the pass, with the
// sample (within the tile) its amplitudes belong to under the current mapping.
template <int NT>
__device__ __forceinline__ void grad_record(float* gacc, uint8_t* gsmp, int rel, int tid, float g, int sample_off) {
    gacc[rel * NT + tid] = g;
    gsmp[rel * NT + tid] = (uint8_t)sample_off;
}

// Exchange psi and lambda through their buffers to the mapping (y, z, w).
template <int TB, int RB>
__device__ __forceinline__ void exchange2(PTile<RB>& pt, PTile<RB>& lt, uint32_t& xm, ThreadMap& tm, float* pp,
                                          float* lp, const PassDesc& d, int32_t y, int32_t z, int32_t w, int tid,
                                          uint32_t fixed_val) {
    cta_sync<(1 << (TB - RB))>();
    const int base = tm.sw_base ^ xm_slot_offset<RB>(tm, xm);
    pxwrite_k<RB>(pp, pt, tm, base, 1 << TB);
    pxwrite_k<RB>(lp, lt, tm, base, 1 << TB);
    xm = 0;
    cta_sync<(1 << (TB - RB))>();
    decode_map<RB>(d, y, z, w, tid, fixed_val, tm);
    pxread_k<RB>(pp, pt, tm, 1 << TB);
    pxread_k<RB>(lp, lt, tm, 1 << TB);
}

// The backward's producer warp.  Tile i of the CTA uses slot i % 2 (psi and
// lambda buffers); the warp stores tile i - 2 out of the slot once the
// compute warps released it (the psi and lambda the pass updates), waits
// until the bulk copies have read the slot, then publishes tile i's geometry
// and loads its psi and lambda with bulk copies that complete on the slot's
// full barrier.  Blocks of 2^cb contiguous amplitudes as in the forward.
template <int TB>
__device__ __forceinline__ void bwd_producer(const PassDesc& d, const RunArgs& A, const float2* psi_src,
                                             bool store_psi, bool store_lam, int64_t num_tiles, float2* pbuf0,
                                             uint64_t* bar_full, uint64_t* bar_empty, TileGeo* s_geo, int lane) {
    constexpr int AMPS = 1 << TB;
    constexpr int KB = ((1 << (TB - 6)) + 31) / 32;  // cached block offsets per lane
    const int n = A.n;
    const bool whole = n < TB;
    int cb = d.run_bits;
    while (cb < TB && d.gbit[cb] == cb) ++cb;
    const int nblk = 1 << (TB - cb);
    const uint32_t bbytes = 8u << cb;
    auto block_off = [&](int b) {
        uint32_t o = 0;
        for (int k = 0; k < TB - cb; ++k)
            if ((b >> k) & 1) o |= 1u << d.gbit[cb + k];
        return o;
    };
    uint32_t off[KB];
#pragma unroll
    for (int k = 0; k < KB; ++k) off[k] = lane + 32 * k < nblk ? block_off(lane + 32 * k) : 0;
    const uint32_t fmask = fixed_mask_of(d);
    const int64_t G = gridDim.x;
    const int64_t t0 = blockIdx.x;
    const int64_t mine = (num_tiles - t0 + G - 1) / G;
    bool failed = false;
    int64_t failed_tile = -1;
    for (int64_t i = 0; i < mine + 2; ++i) {
        const int s = (int)(i & 1);
        float2* ps = pbuf0 + s * 2 * AMPS;
        float2* ls = ps + AMPS;
        if (i >= 2) {
            // the lanes agree before any of them leaves the loop: a lane that
            // gave up alone would miss the warp-wide __syncwarp and
            // __reduce_add_sync below
            const bool released = mbar_wait(bar_empty + s, (uint32_t)((i / 2 - 1) & 1));
            if (!__all_sync(0xffffffffu, released)) {
                failed = true;
                failed_tile = t0 + (i - 2) * G;
                break;
            }
            if (store_psi || store_lam) {
                const TileGeo g = tile_geo_m(TB, fmask, t0 + (i - 2) * G, n, A.batch);
                if (whole) {
                    if (lane == 0) {
                        const uint32_t bytes = (uint32_t)(((int64_t)g.nsamples << n) * 8);
                        if (store_psi) bulk_s2g(A.state + g.base, ps, bytes);
                        if (store_lam) bulk_s2g(A.lam + g.base, ls, bytes);
                    }
                } else {
                    for (int b = lane, k = 0; b < nblk; b += 32, ++k) {
                        const uint32_t o = k < KB ? off[k < KB ? k : 0] : block_off(b);
                        if (store_psi) bulk_s2g(A.state + g.base + o, ps + ((int64_t)b << cb), bbytes);
                        if (store_lam) bulk_s2g(A.lam + g.base + o, ls + ((int64_t)b << cb), bbytes);
                    }
                }
                bulk_commit();
                bulk_wait_read0();  // this lane's copies have read the slot
            }
            __syncwarp();  // every copy out of the slot has read it
        }
        if (i < mine) {
            const TileGeo g = tile_geo_m(TB, fmask, t0 + i * G, n, A.batch);
            if (lane == 0) s_geo[s] = g;  // published by lane 0's arrive below
            uint32_t bytes = 0;
            if (whole) {
                if (lane == 0) bytes = 2u * (uint32_t)(((int64_t)g.nsamples << n) * 8);
            } else {
                for (int b = lane; b < nblk; b += 32) bytes += 2u * bbytes;
            }
            const uint32_t warp_bytes = __reduce_add_sync(0xffffffffu, bytes);
            if (lane == 0) mbar_arrive_expect_tx(bar_full + s, warp_bytes);
            __syncwarp();
            if (whole) {
                if (lane == 0) {
                    bulk_g2s(ps, psi_src + g.base, bytes / 2, bar_full + s);
                    bulk_g2s(ls, A.lam + g.base, bytes / 2, bar_full + s);
                }
            } else {
                for (int b = lane, k = 0; b < nblk; b += 32, ++k) {
                    const uint32_t o = k < KB ? off[k < KB ? k : 0] : block_off(b);
                    bulk_g2s(ps + ((int64_t)b << cb), psi_src + g.base + o, bbytes, bar_full + s);
                    bulk_g2s(ls + ((int64_t)b << cb), A.lam + g.base + o, bbytes, bar_full + s);
                }
            }
        }
    }
    bulk_wait_all0();  // this lane's stores have completed before it leaves
    if (failed && lane == 0) report_timeout(A.status, kSiteBwdProducer, failed_tile);
}

// Body of the backward pass kernel: psi and lambda tiles, gradient partials.
// The CTA's last warp is the producer (bwd_producer); the compute warps wait
// for a slot, run Ops::apply on the thread's two tiles (shared pending X,
// recording gradient partials into gacc / gsmp), reduce the partials per
// sample in a fixed order, write psi and lambda back into the slot and
// release it.
template <int TB, int RB, class Ops>
__device__ __forceinline__ void bwd_pass_body(const PassDesc* __restrict__ passes, const int4* __restrict__ ops_all,
                                              int pass_index, const RunArgs& A, int store_lam_last,
                                              int64_t num_tiles) {
    constexpr int NT = 1 << (TB - RB);
    constexpr int AMPS = 1 << TB;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float2* pbuf0 = reinterpret_cast<float2*>(smem_raw);  // slot 0: psi, lambda; slot 1: psi, lambda
    int4* s_ops = reinterpret_cast<int4*>(pbuf0 + 4 * AMPS);         // [kSmemOps]
    float4* s_mats = reinterpret_cast<float4*>(s_ops + kSmemOps);     // [kSmemMats][2]
    float* gacc = reinterpret_cast<float*>(s_mats + 2 * kSmemMats);  // [ngrad][NT]
    // sample (within the tile) each partial belongs to: the thread's sample
    // bits depend on the mapping in force when the gradient op ran
    uint8_t* gsmp = reinterpret_cast<uint8_t*>(gacc + max_grad_per_pass(RB) * NT);  // [ngrad][NT]
    uint64_t* bar_full = reinterpret_cast<uint64_t*>(gsmp + max_grad_per_pass(RB) * NT);  // [2]
    uint64_t* bar_empty = bar_full + 2;                                                   // [2]
    __shared__ PassDesc sd;
    __shared__ TileGeo s_geo[2];

    const int tid = threadIdx.x;
    if (tid == 0) {
        sd = passes[pass_index];
        for (int s = 0; s < 2; ++s) {
            mbar_init(bar_full + s, 1);        // the producer's lane 0 (with the copies' bytes)
            mbar_init(bar_empty + s, NT / 32);  // lane 0 of every compute warp
        }
    }
    __syncthreads();  // the only barrier the producer joins
    const PassDesc& d = sd;
    const int n = A.n;
    const float2* psi_src = d.psi_from_ckpt >= 0 ? A.ckpt + (int64_t)d.psi_from_ckpt * (A.batch << n) : A.state;
    const bool store_psi = (d.epi & EPI_STORE) != 0;
    const bool store_lam = store_psi || store_lam_last;
    if (tid >= NT) {
        bwd_producer<TB>(d, A, psi_src, store_psi, store_lam, num_tiles, pbuf0, bar_full, bar_empty, s_geo,
                         tid - NT);
        return;
    }
    const int4* ops = ops_all + d.op_begin;
    if (Ops::kStageOps)
        for (int i = tid; i < d.op_count && i < kSmemOps; i += NT) s_ops[i] = __ldg(ops + i);
    {
        const int nm = A.nslots_shared < kSmemMats ? A.nslots_shared : kSmemMats;
        const float4* gm = reinterpret_cast<const float4*>(A.mats);
        for (int i = tid; i < 2 * nm; i += NT) s_mats[i] = __ldg(gm + i);
    }
    cta_sync<NT>();
    int iter = 0;
    bool ok = true;
    int64_t failed_tile = -1;
    for (int64_t t = blockIdx.x; t < num_tiles; t += gridDim.x, ++iter) {
        const int slot = iter & 1;
        float2* ps = pbuf0 + slot * 2 * AMPS;
        float2* ls = ps + AMPS;
        const bool landed = mbar_wait(bar_full + slot, (uint32_t)((iter >> 1) & 1));
        if (!cta_sync_and<NT>(landed)) {
            ok = false;
            failed_tile = t;
            break;
        }
        const TileGeo g = s_geo[slot];
        PTile<RB> pt, lt;
        uint32_t xm = 0;  // pending thread-controlled X, shared by psi and lambda
        ThreadMap tm;
        pload_nat<RB>(pt, ps, tid);
        pload_nat<RB>(lt, ls, tid);
        decode_map<RB>(d, NatMap<TB, RB>::y, NatMap<TB, RB>::z, NatMap<TB, RB>::w, tid, g.fixed_val, tm);
        Ops::template apply<TB, RB>(pt, lt, xm, tm, d, A, ops, s_ops, s_mats, reinterpret_cast<float*>(ps),
                                    reinterpret_cast<float*>(ls), g.sample, g.fixed_val, tid, gacc, gsmp);
        cta_sync<NT>();  // exchange reads of the slot and every gradient partial are done
        // gradient partials of this tile: per sample when samples share the tile
        if (d.ngrad > 0) {
            const int nq = d.nq_tile;
            const int spt = (nq < TB) ? (1 << (TB - nq)) : 1;
            const int64_t tps = (n >= TB) ? (int64_t(1) << (n - TB)) : 1;
            const int64_t units = (n >= TB) ? A.batch * tps : A.batch;
            const int items = d.ngrad * spt;
            const int warp = tid >> 5, lane = tid & 31;
            for (int it = warp; it < items; it += NT / 32) {
                int gi = it / spt, s = it % spt;
                float acc = 0.f;
                for (int c = lane; c < NT; c += 32)
                    if (gsmp[gi * NT + c] == s) acc += gacc[gi * NT + c];
                for (int o2 = 16; o2 > 0; o2 >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o2);
                if (lane == 0 && s < g.nsamples) {
                    int64_t unit = (n >= TB) ? (g.sample * tps + g.tile_in_sample) : (g.sample + s);
                    A.gradpart[(int64_t)(d.grad_base + gi) * units + unit] = acc;
                }
            }
        }
        // psi and lambda (natural mapping) back into the slot for the producer
        if (store_psi) pstore_nat<RB>(pt, ps, tid, xm);
        if (store_lam) pstore_nat<RB>(lt, ls, tid, xm);
        fence_proxy_async();
        __syncwarp();
        if ((tid & 31) == 0) mbar_arrive(bar_empty + slot);
    }
    if (!ok && tid == 0) report_timeout(A.status, kSiteBwdCompute, failed_tile);
}

}  // namespace qg

// Backward (adjoint) pass kernel shared by the prebuilt op interpreter
// (fused.cu) and the backward pass kernels compiled at run time (jit.cpp).
// Device code only, handed to NVRTC as text.
//
// A backward pass walks tiles of psi (the state) and lambda (the cotangent):
// both arrive by per-thread async copies into a double buffer, the pass's
// inverse gates act on both in registers with one shared pending-X mask, and
// every rotation first leaves its gradient partial Im<lambda|P|psi> in shared
// memory; the partials of a tile are reduced per sample in a fixed order.
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
    __syncthreads();
    const int base = tm.sw_base ^ xm_slot_offset<RB>(tm, xm);
    pxwrite_k<RB>(pp, pt, tm, base, 1 << TB);
    pxwrite_k<RB>(lp, lt, tm, base, 1 << TB);
    xm = 0;
    __syncthreads();
    decode_map<RB>(d, y, z, w, tid, fixed_val, tm);
    pxread_k<RB>(pp, pt, tm, 1 << TB);
    pxread_k<RB>(lp, lt, tm, 1 << TB);
}

// Body of the backward pass kernel: psi and lambda tiles, gradient
// partials.  Ops::apply runs the pass's gate program on the thread's two
// tiles (shared pending X), recording gradient partials into gacc / gsmp.
template <int TB, int RB, class Ops>
__device__ __forceinline__ void bwd_pass_body(const PassDesc* __restrict__ passes, const int4* __restrict__ ops_all,
                                              int pass_index, const RunArgs& A, int store_lam_last,
                                              int64_t num_tiles) {
    constexpr int NT = 1 << (TB - RB);
    constexpr int AMPS = 1 << TB;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float2* pbuf0 = reinterpret_cast<float2*>(smem_raw);  // psi, lambda, psi, lambda
    int4* s_ops = reinterpret_cast<int4*>(pbuf0 + 4 * AMPS);         // [kSmemOps]
    float4* s_mats = reinterpret_cast<float4*>(s_ops + kSmemOps);     // [kSmemMats][2]
    float* gacc = reinterpret_cast<float*>(s_mats + 2 * kSmemMats);  // [ngrad][NT]
    // sample (within the tile) each partial belongs to: the thread's sample
    // bits depend on the mapping in force when the gradient op ran
    uint8_t* gsmp = reinterpret_cast<uint8_t*>(gacc + max_grad_per_pass(RB) * NT);  // [ngrad][NT]
    __shared__ PassDesc sd;

    const int tid = threadIdx.x;
    if (tid == 0) sd = passes[pass_index];
    __syncthreads();
    const PassDesc& d = sd;
    const int4* ops = ops_all + d.op_begin;
    if (Ops::kStageOps)
        for (int i = tid; i < d.op_count && i < kSmemOps; i += NT) s_ops[i] = __ldg(ops + i);
    {
        const int nm = A.nslots_shared < kSmemMats ? A.nslots_shared : kSmemMats;
        const float4* gm = reinterpret_cast<const float4*>(A.mats);
        for (int i = tid; i < 2 * nm; i += NT) s_mats[i] = __ldg(gm + i);
    }
    const int n = A.n;
    const float2* psi_src = d.psi_from_ckpt >= 0 ? A.ckpt + (int64_t)d.psi_from_ckpt * (A.batch << n) : A.state;
    const bool last = (d.epi & EPI_STORE) == 0;  // final backward pass: nothing to store but lambda
    (void)last;

    __syncthreads();
    // psi and lambda of a tile arrive as one cp.async group per thread; every
    // thread commits one group per tile (empty past the last tile), so
    // "tile t has landed" is wait_group 0 before the next commit + a barrier
    auto prefetch = [&](int64_t t, float2* dst) {
        if (t < num_tiles) {
            TileGeo gn = tile_geo(d, t, n, A.batch);
            thread_tile_load<TB, RB>(d, gn, psi_src, dst, n, tid);
            thread_tile_load<TB, RB>(d, gn, A.lam, dst + AMPS, n, tid);
        }
        cp_async_commit();
    };
    int64_t t0 = blockIdx.x;
    prefetch(t0, pbuf0);
    int iter = 0;
    for (int64_t t = t0; t < num_tiles; t += gridDim.x, ++iter) {
        float2* ps = pbuf0 + (iter & 1) * 2 * AMPS;
        float2* ls = ps + AMPS;
        float2* nps = pbuf0 + ((iter + 1) & 1) * 2 * AMPS;
        TileGeo g = tile_geo(d, t, n, A.batch);
        PTile<RB> pt, lt;
        uint32_t xm = 0;  // pending thread-controlled X, shared by psi and lambda
        ThreadMap tm;
        cp_async_wait<0>();
        __syncthreads();
        pload_nat<RB>(pt, ps, tid);
        pload_nat<RB>(lt, ls, tid);
        decode_map<RB>(d, NatMap<TB, RB>::y, NatMap<TB, RB>::z, NatMap<TB, RB>::w, tid, g.fixed_val, tm);
        // the other buffer pair held tile t - 1, whose end waited for every read
        prefetch(t + gridDim.x, nps);
        Ops::template apply<TB, RB>(pt, lt, xm, tm, d, A, ops, s_ops, s_mats, reinterpret_cast<float*>(ps),
                                    reinterpret_cast<float*>(ls), g.sample, g.fixed_val, tid, gacc, gsmp);
        __syncthreads();
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
        // store psi and lambda (natural mapping) straight from registers
        if (d.epi & EPI_STORE) {
            pstore_global<RB>(pt, xm, d, g, A.state, n, tid);
            pstore_global<RB>(lt, xm, d, g, A.lam, n, tid);
        } else if (store_lam_last) {
            pstore_global<RB>(lt, xm, d, g, A.lam, n, tid);
        }
        __syncthreads();  // `ps` / `ls` are free for the prefetch two tiles ahead
    }
    cp_async_wait<0>();
}

}  // namespace qg

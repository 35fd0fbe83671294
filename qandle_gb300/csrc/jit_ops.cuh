// Gate ops with compile-time register positions, called by the pass kernels
// that jit.cpp generates for one program and compiles with NVRTC.
//
// The op interpreter (fused.cu) dispatches every op on its runtime register
// position; here the position is a template argument, so a CNOT or SWAP
// between register qubits is a renaming of registers that costs no
// instruction, and consecutive gates on different qubits interleave freely.
//
// Pending X (planar.cuh): physical register r holds logical amplitude
// r ^ xm.  The rules below keep xm exact without moving data:
//   CX(c -> p), both in registers: apply the physical CX and set
//     xm_p ^= xm_c  (X_c CX X_c = X_p CX);
//   SWAP(a, b): apply the physical SWAP and swap bits a and b of xm;
//   a matrix on bit p with xm_p set acts as X M X (rows and columns reversed).
#pragma once
#include "bwd_kernel.cuh"

namespace qg {

// X M X of a row-form 2x2 where c holds, else M.
__device__ __forceinline__ void xmx_if(float2 m[4], bool c) {
    const float2 a = m[0], b = m[1], e = m[2], f = m[3];
    m[0] = c ? f : a;
    m[1] = c ? e : b;
    m[2] = c ? b : e;
    m[3] = c ? a : f;
}

template <int P, int RB>
__device__ __forceinline__ void jmat(PTile<RB>& pt, uint32_t xm, const RunArgs& A, const float4* s_mats, int slot,
                                     int flags, int64_t sample) {
    float2 m[4];
    load_slot(A, s_mats, slot, flags, sample, m);
    xmx_if(m, (xm >> P) & 1u);
    pmat<P, RB>(pt, m);
}

// A matrix staged in shared memory (two float4: M00 M01 | M10 M11).
__device__ __forceinline__ void smem_mat(const float4* sm, float2 m[4]) {
    const float4 u = sm[0], v = sm[1];
    m[0] = make_float2(u.x, u.y);
    m[1] = make_float2(u.z, u.w);
    m[2] = make_float2(v.x, v.y);
    m[3] = make_float2(v.z, v.w);
}

// Per-sample matrix k of the tile's sample, staged at the tile's start.
template <int P, int RB>
__device__ __forceinline__ void jmat_staged(PTile<RB>& pt, uint32_t xm, const float4* staged, int k) {
    float2 m[4];
    smem_mat(staged + 2 * k, m);
    xmx_if(m, (xm >> P) & 1u);
    pmat<P, RB>(pt, m);
}

template <int P, int RB>
__device__ __forceinline__ void jdiag_staged(PTile<RB>& pt, uint32_t xm, const float4* staged, int k) {
    float2 m[4];
    smem_mat(staged + 2 * k, m);
    const bool sw = (xm >> P) & 1u;
    pdiag<P, RB>(pt, sw ? m[3] : m[0], sw ? m[0] : m[3]);
}

template <int RB>
__device__ __forceinline__ void jdiag_thread_staged(PTile<RB>& pt, bool bit, const float4* staged, int k) {
    float2 m[4];
    smem_mat(staged + 2 * k, m);
    pscale<RB>(pt, bit ? m[3] : m[0]);
}

template <int P, int RB>
__device__ __forceinline__ void jdiag(PTile<RB>& pt, uint32_t xm, const RunArgs& A, const float4* s_mats, int slot,
                                      int flags, int64_t sample) {
    float2 m[4];
    load_slot(A, s_mats, slot, flags, sample, m);
    const bool sw = (xm >> P) & 1u;
    pdiag<P, RB>(pt, sw ? m[3] : m[0], sw ? m[0] : m[3]);
}

// Diagonal on a thread-uniform bit: one complex factor for the whole thread.
template <int RB>
__device__ __forceinline__ void jdiag_thread(PTile<RB>& pt, bool bit, const RunArgs& A, const float4* s_mats,
                                             int slot, int flags, int64_t sample) {
    float2 m[4];
    load_slot(A, s_mats, slot, flags, sample, m);
    pscale<RB>(pt, bit ? m[3] : m[0]);
}

template <int P, int C, int RB>
__device__ __forceinline__ void jcx(PTile<RB>& pt, uint32_t& xm) {
    pcx<P, C, RB>(pt);
    xm ^= ((xm >> C) & 1u) << P;
}

template <int P0, int P1, int RB>
__device__ __forceinline__ void jswap(PTile<RB>& pt, uint32_t& xm) {
    pswapbits<P0, P1, RB>(pt);
    const uint32_t d = ((xm >> P0) ^ (xm >> P1)) & 1u;
    xm ^= d * ((1u << P0) | (1u << P1));
}

// Apply the pending X of register bit P and clear it.
template <int P, int RB>
__device__ __forceinline__ void jmaterialize(PTile<RB>& pt, uint32_t& xm) {
    pswap_if<P, RB>(pt, (xm >> P) & 1u);
    xm &= ~(1u << P);
}

// Negate the amplitudes whose register bits in Mask are all 1, where c holds
// (a per-thread condition: a sign multiply instead of a divergent branch).
template <int Mask, int RB>
__device__ __forceinline__ void jnegate_if(PTile<RB>& pt, bool c) {
    const float s = c ? -1.f : 1.f;
#pragma unroll
    for (int r = 0; r < (1 << RB); ++r) {
        if ((r & Mask) != Mask) continue;
        const float2 a = get_amp<RB>(pt, r);
        set_amp<RB>(pt, r, make_float2(a.x * s, a.y * s));
    }
}

// ---- exchanges with compile-time slot offsets ----
//
// The swizzle (fwd_kernel.cuh, swz) is linear over XOR, so the shared-memory
// slot of a thread's register amplitude K under a mapping is
// base ^ XOR_{bits k of K} C_k, where base depends on the thread's lane/warp
// bits only and C_k = swz(1 << local bit of register bit k).  The generated
// pass knows every mapping, so the C_k are template arguments.

template <int K, int C0, int C1, int C2, int C3, int C4>
__device__ __forceinline__ constexpr int kxor() {
    return ((K & 1) ? C0 : 0) ^ ((K & 2) ? C1 : 0) ^ ((K & 4) ? C2 : 0) ^ ((K & 8) ? C3 : 0) ^ ((K & 16) ? C4 : 0);
}

template <int C0, int C1, int C2, int C3, int C4>
__device__ __forceinline__ int xm_xor(uint32_t xm) {
    return ((xm & 1u) ? C0 : 0) ^ ((xm & 2u) ? C1 : 0) ^ ((xm & 4u) ? C2 : 0) ^ ((xm & 8u) ? C3 : 0) ^
           ((xm & 16u) ? C4 : 0);
}

template <int TB, int RB, int C0, int C1, int C2, int C3, int C4, int K = 0>
__device__ __forceinline__ void cxwrite(float* plane, const PTile<RB>& t, int base) {
    const int s = base ^ kxor<K, C0, C1, C2, C3, C4>();
    const float2 a = get_amp<RB>(t, K);
    plane[s] = a.x;
    plane[s + (1 << TB)] = a.y;
    if constexpr (K + 1 < (1 << RB)) cxwrite<TB, RB, C0, C1, C2, C3, C4, K + 1>(plane, t, base);
}

template <int TB, int RB, int C0, int C1, int C2, int C3, int C4, int K = 0>
__device__ __forceinline__ void cxread(const float* plane, PTile<RB>& t, int base) {
    const int s = base ^ kxor<K, C0, C1, C2, C3, C4>();
    set_amp<RB>(t, K, make_float2(plane[s], plane[s + (1 << TB)]));
    if constexpr (K + 1 < (1 << RB)) cxread<TB, RB, C0, C1, C2, C3, C4, K + 1>(plane, t, base);
}

// Thread bit k of the thread index as 0/1.
__device__ __forceinline__ int tbit(int tid, int k) { return (tid >> k) & 1; }

// ---- backward: the same ops on psi and lambda (one pending-X mask) ----

template <int P, int RB>
__device__ __forceinline__ void jmat2(PTile<RB>& pt, PTile<RB>& lt, uint32_t xm, const RunArgs& A,
                                      const float4* s_mats, int slot, int flags, int64_t sample) {
    float2 m[4];
    load_slot(A, s_mats, slot, flags, sample, m);
    xmx_if(m, (xm >> P) & 1u);
    pmat<P, RB>(pt, m);
    pmat<P, RB>(lt, m);
}

template <int P, int RB>
__device__ __forceinline__ void jdiag2(PTile<RB>& pt, PTile<RB>& lt, uint32_t xm, const RunArgs& A,
                                       const float4* s_mats, int slot, int flags, int64_t sample) {
    float2 m[4];
    load_slot(A, s_mats, slot, flags, sample, m);
    const bool sw = (xm >> P) & 1u;
    const float2 d0 = sw ? m[3] : m[0], d1 = sw ? m[0] : m[3];
    pdiag<P, RB>(pt, d0, d1);
    pdiag<P, RB>(lt, d0, d1);
}

template <int RB>
__device__ __forceinline__ void jdiag_thread2(PTile<RB>& pt, PTile<RB>& lt, bool bit, const RunArgs& A,
                                              const float4* s_mats, int slot, int flags, int64_t sample) {
    float2 m[4];
    load_slot(A, s_mats, slot, flags, sample, m);
    pscale<RB>(pt, bit ? m[3] : m[0]);
    pscale<RB>(lt, bit ? m[3] : m[0]);
}

template <int P, int C, int RB>
__device__ __forceinline__ void jcx2(PTile<RB>& pt, PTile<RB>& lt, uint32_t& xm) {
    pcx<P, C, RB>(pt);
    pcx<P, C, RB>(lt);
    xm ^= ((xm >> C) & 1u) << P;
}

template <int P0, int P1, int RB>
__device__ __forceinline__ void jswap2(PTile<RB>& pt, PTile<RB>& lt, uint32_t& xm) {
    pswapbits<P0, P1, RB>(pt);
    pswapbits<P0, P1, RB>(lt);
    const uint32_t d = ((xm >> P0) ^ (xm >> P1)) & 1u;
    xm ^= d * ((1u << P0) | (1u << P1));
}

template <int P, int RB>
__device__ __forceinline__ void jmaterialize2(PTile<RB>& pt, PTile<RB>& lt, uint32_t& xm) {
    const bool c = (xm >> P) & 1u;
    pswap_if<P, RB>(pt, c);
    pswap_if<P, RB>(lt, c);
    xm &= ~(1u << P);
}

template <int Mask, int RB>
__device__ __forceinline__ void jnegate2(PTile<RB>& pt, PTile<RB>& lt) {
    pnegate<Mask, RB>(pt);
    pnegate<Mask, RB>(lt);
}

template <int Mask, int RB>
__device__ __forceinline__ void jnegate_if2(PTile<RB>& pt, PTile<RB>& lt, bool c) {
    jnegate_if<Mask, RB>(pt, c);
    jnegate_if<Mask, RB>(lt, c);
}

// Gradient partial of the rotation on register bit P (axis of its generator)
// into grad slot `rel` of the pass.
template <int P, int RB, int NT>
__device__ __forceinline__ void jgrad(const PTile<RB>& pt, const PTile<RB>& lt, uint32_t xm, int axis, float* gacc,
                                      uint8_t* gsmp, int rel, int tid, int sample_off) {
    grad_record<NT>(gacc, gsmp, rel, tid, pgrad_at<P, RB>(pt, lt, axis, xm), sample_off);
}

}  // namespace qg

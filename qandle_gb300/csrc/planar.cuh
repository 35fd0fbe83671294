// Planar register tiles for the forward pass kernel.
//
// A thread holds 2^RB amplitudes.  Amplitude r keeps its real part in
// R[r >> 1] and its imaginary part in I[r >> 1], lane .x for even r and .y for
// odd r.  One 64-bit register pair therefore holds the same part of the two
// amplitudes that differ in register bit 0, and the Blackwell packed FP32
// instructions (fma.rn.f32x2 / mul.rn.f32x2) update both with one issue.  A
// complex 2x2 on a register qubit costs 4 packed instructions per amplitude
// instead of 8 scalar FMAs.
//
// Pending X: a CNOT whose control is a thread-uniform bit (lane, warp or a
// qubit outside the tile) and whose target is register bit p is not applied
// by moving data.  The thread records it in `xm` (physical register r then
// holds logical amplitude r ^ xm), later ops on p use the conjugated matrix
// X M X, and the next exchange or store writes every register to the slot of
// its logical index, which costs one XOR per thread.
#pragma once
#include "devmath.cuh"

namespace qg {

__device__ __forceinline__ unsigned long long pk2(float2 v) { return *reinterpret_cast<unsigned long long*>(&v); }
__device__ __forceinline__ float2 upk2(unsigned long long u) { return *reinterpret_cast<float2*>(&u); }

// a * b + c on both lanes
__device__ __forceinline__ float2 vfma(float2 a, float2 b, float2 c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pk2(a)), "l"(pk2(b)), "l"(pk2(c)));
    return upk2(r);
}
__device__ __forceinline__ float2 vmul(float2 a, float2 b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(r);
}
__device__ __forceinline__ float2 bcast(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 lswap(float2 v) { return make_float2(v.y, v.x); }
__device__ __forceinline__ float2 vsel(bool c, float2 a, float2 b) { return c ? a : b; }

template <int RB>
struct PTile {
    static constexpr int H = 1 << (RB - 1);
    float2 R[H], I[H];
};

template <int RB>
__device__ __forceinline__ float2 get_amp(const PTile<RB>& t, int r) {
    return (r & 1) ? make_float2(t.R[r >> 1].y, t.I[r >> 1].y) : make_float2(t.R[r >> 1].x, t.I[r >> 1].x);
}
template <int RB>
__device__ __forceinline__ void set_amp(PTile<RB>& t, int r, float2 a) {
    if (r & 1) {
        t.R[r >> 1].y = a.x;
        t.I[r >> 1].y = a.y;
    } else {
        t.R[r >> 1].x = a.x;
        t.I[r >> 1].x = a.y;
    }
}

// Row-form 2x2 (out = in @ M) on register bit P.  m[0..3] = M00 M01 M10 M11.
template <int P, int RB>
__device__ __forceinline__ void pmat(PTile<RB>& t, const float2 m[4]) {
    constexpr int H = 1 << (RB - 1);
    if constexpr (P == 0) {
        // lanes x / y of one vector are the pair: o_x = M00 a_x + M10 a_y, o_y = M01 a_x + M11 a_y
        const float2 cAr = make_float2(m[0].x, m[3].x), cAi = make_float2(m[0].y, m[3].y);
        const float2 cBr = make_float2(m[2].x, m[1].x), cBi = make_float2(m[2].y, m[1].y);
        const float2 nAi = make_float2(-cAi.x, -cAi.y), nBi = make_float2(-cBi.x, -cBi.y);
#pragma unroll
        for (int k = 0; k < H; ++k) {
            const float2 r = t.R[k], i = t.I[k], rs = lswap(r), is = lswap(i);
            float2 nr = vmul(cAr, r);
            nr = vfma(nAi, i, nr);
            nr = vfma(cBr, rs, nr);
            nr = vfma(nBi, is, nr);
            float2 ni = vmul(cAr, i);
            ni = vfma(cAi, r, ni);
            ni = vfma(cBr, is, ni);
            ni = vfma(cBi, rs, ni);
            t.R[k] = nr;
            t.I[k] = ni;
        }
    } else {
        constexpr int Q = 1 << (P - 1);
        const float2 c00r = bcast(m[0].x), c00i = bcast(m[0].y), n00i = bcast(-m[0].y);
        const float2 c01r = bcast(m[1].x), c01i = bcast(m[1].y), n01i = bcast(-m[1].y);
        const float2 c10r = bcast(m[2].x), c10i = bcast(m[2].y), n10i = bcast(-m[2].y);
        const float2 c11r = bcast(m[3].x), c11i = bcast(m[3].y), n11i = bcast(-m[3].y);
#pragma unroll
        for (int k = 0; k < H; ++k) {
            if (k & Q) continue;
            const float2 r0 = t.R[k], i0 = t.I[k], r1 = t.R[k | Q], i1 = t.I[k | Q];
            float2 a = vmul(c00r, r0);
            a = vfma(n00i, i0, a);
            a = vfma(c10r, r1, a);
            a = vfma(n10i, i1, a);
            float2 b = vmul(c00r, i0);
            b = vfma(c00i, r0, b);
            b = vfma(c10r, i1, b);
            b = vfma(c10i, r1, b);
            float2 c = vmul(c01r, r0);
            c = vfma(n01i, i0, c);
            c = vfma(c11r, r1, c);
            c = vfma(n11i, i1, c);
            float2 d = vmul(c01r, i0);
            d = vfma(c01i, r0, d);
            d = vfma(c11r, i1, d);
            d = vfma(c11i, r1, d);
            t.R[k] = a;
            t.I[k] = b;
            t.R[k | Q] = c;
            t.I[k | Q] = d;
        }
    }
}

// Diagonal diag(d0, d1) on register bit P.
template <int P, int RB>
__device__ __forceinline__ void pdiag(PTile<RB>& t, float2 d0, float2 d1) {
    constexpr int H = 1 << (RB - 1);
#pragma unroll
    for (int k = 0; k < H; ++k) {
        float2 dr, di;
        if constexpr (P == 0) {
            dr = make_float2(d0.x, d1.x);
            di = make_float2(d0.y, d1.y);
        } else {
            const float2 d = (k & (1 << (P - 1))) ? d1 : d0;
            dr = bcast(d.x);
            di = bcast(d.y);
        }
        const float2 r = t.R[k], i = t.I[k];
        t.R[k] = vfma(make_float2(-di.x, -di.y), i, vmul(dr, r));
        t.I[k] = vfma(di, r, vmul(dr, i));
    }
}

// One complex factor on every amplitude.
template <int RB>
__device__ __forceinline__ void pscale(PTile<RB>& t, float2 d) {
    constexpr int H = 1 << (RB - 1);
    const float2 dr = bcast(d.x), di = bcast(d.y), ndi = bcast(-d.y);
#pragma unroll
    for (int k = 0; k < H; ++k) {
        const float2 r = t.R[k], i = t.I[k];
        t.R[k] = vfma(ndi, i, vmul(dr, r));
        t.I[k] = vfma(di, r, vmul(dr, i));
    }
}

// Exchange the amplitudes of register bit P pairs where `c` holds (thread-uniform).
template <int P, int RB>
__device__ __forceinline__ void pswap_if(PTile<RB>& t, bool c) {
    constexpr int H = 1 << (RB - 1);
    if constexpr (P == 0) {
#pragma unroll
        for (int k = 0; k < H; ++k) {
            t.R[k] = vsel(c, lswap(t.R[k]), t.R[k]);
            t.I[k] = vsel(c, lswap(t.I[k]), t.I[k]);
        }
    } else {
        constexpr int Q = 1 << (P - 1);
#pragma unroll
        for (int k = 0; k < H; ++k) {
            if (k & Q) continue;
            const float2 r0 = t.R[k], r1 = t.R[k | Q], i0 = t.I[k], i1 = t.I[k | Q];
            t.R[k] = vsel(c, r1, r0);
            t.R[k | Q] = vsel(c, r0, r1);
            t.I[k] = vsel(c, i1, i0);
            t.I[k | Q] = vsel(c, i0, i1);
        }
    }
}

// X on register bit P where register bit C is 1 (a fixed permutation).
template <int P, int C, int RB>
__device__ __forceinline__ void pcx(PTile<RB>& t) {
    constexpr int N = 1 << RB;
#pragma unroll
    for (int r = 0; r < N; ++r) {
        if ((r & (1 << P)) || !(r & (1 << C))) continue;
        const float2 a = get_amp<RB>(t, r), b = get_amp<RB>(t, r | (1 << P));
        set_amp<RB>(t, r, b);
        set_amp<RB>(t, r | (1 << P), a);
    }
}

// Exchange register bits P0 and P1 (SWAP of two register qubits).
template <int P0, int P1, int RB>
__device__ __forceinline__ void pswapbits(PTile<RB>& t) {
    constexpr int N = 1 << RB;
#pragma unroll
    for (int r = 0; r < N; ++r) {
        if (!((r & (1 << P0)) && !(r & (1 << P1)))) continue;
        const int s = r ^ (1 << P0) ^ (1 << P1);
        const float2 a = get_amp<RB>(t, r), b = get_amp<RB>(t, s);
        set_amp<RB>(t, r, b);
        set_amp<RB>(t, s, a);
    }
}

// Negate the amplitudes whose register bits in `Mask` are all 1 (compile-time).
template <int Mask, int RB>
__device__ __forceinline__ void pnegate(PTile<RB>& t) {
    constexpr int N = 1 << RB;
#pragma unroll
    for (int r = 0; r < N; ++r) {
        if ((r & Mask) != Mask) continue;
        float2 a = get_amp<RB>(t, r);
        set_amp<RB>(t, r, make_float2(-a.x, -a.y));
    }
}

}  // namespace qg

namespace qg {

// Im( conj(l0) (P p)_0 + conj(l1) (P p)_1 ) summed over the register-bit-P
// pairs of psi (p) and lambda (l); P is the generator of the rotation axis.
template <int P, int RB>
__device__ __forceinline__ float pgrad(const PTile<RB>& ps, const PTile<RB>& ls, int axis) {
    constexpr int H = 1 << (RB - 1);
    float2 acc = make_float2(0.f, 0.f);
    const float2 one = bcast(1.f), mone = bcast(-1.f);
#pragma unroll
    for (int k = 0; k < H; ++k) {
        float2 p0r, p0i, p1r, p1i, l0r, l0i, l1r, l1i;
        if constexpr (P == 0) {
            if (k & 0) continue;
            // pairs are the two lanes of a vector: element 0 = lane x, element 1 = lane y
            p0r = ps.R[k];
            p0i = ps.I[k];
            p1r = lswap(ps.R[k]);
            p1i = lswap(ps.I[k]);
            l0r = ls.R[k];
            l0i = ls.I[k];
            l1r = lswap(ls.R[k]);
            l1i = lswap(ls.I[k]);
            // both lanes hold one pair seen from either side: count each pair once
            // by weighting lane y with 0 below
        } else {
            constexpr int Q = 1 << (P - 1);
            if (k & Q) continue;
            p0r = ps.R[k];
            p0i = ps.I[k];
            p1r = ps.R[k | Q];
            p1i = ps.I[k | Q];
            l0r = ls.R[k];
            l0i = ls.I[k];
            l1r = ls.R[k | Q];
            l1i = ls.I[k | Q];
        }
        float2 g;
        if (axis == AX_X) {
            // l0r p1i - l0i p1r + l1r p0i - l1i p0r
            g = vfma(l0r, p1i, vmul(vmul(l0i, mone), p1r));
            g = vfma(l1r, p0i, g);
            g = vfma(vmul(l1i, mone), p0r, g);
        } else if (axis == AX_Y) {
            // -(l0r p1r + l0i p1i) + (l1r p0r + l1i p0i)
            g = vfma(l1r, p0r, vmul(l1i, p0i));
            g = vfma(vmul(l0r, mone), p1r, g);
            g = vfma(vmul(l0i, mone), p1i, g);
        } else {
            // (l0r p0i - l0i p0r) - (l1r p1i - l1i p1r)
            g = vfma(l0r, p0i, vmul(vmul(l0i, mone), p0r));
            g = vfma(vmul(l1r, mone), p1i, g);
            g = vfma(l1i, p1r, g);
        }
        if constexpr (P == 0) g.y = 0.f;
        acc = vfma(g, one, acc);
    }
    return acc.x + acc.y;
}

}  // namespace qg

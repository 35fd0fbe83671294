// Device arithmetic shared by the prebuilt kernels and by the pass kernels
// compiled at run time (NVRTC): nothing here needs a host header.
#pragma once
#ifdef __CUDACC_RTC__
typedef signed char int8_t;
typedef unsigned char uint8_t;
typedef int int32_t;
typedef unsigned int uint32_t;
typedef long long int64_t;
typedef unsigned long long uint64_t;
#else
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#endif

namespace qg {

// device-side copy of QG_ETIMEOUT (a bounded wait gave up)
constexpr int kStatusTimeout = 3;

// Rotation axes, in the order of utils.parse_rot (qandle/utils.py:26-37).
enum Axis : int { AX_X = 0, AX_Y = 1, AX_Z = 2 };

__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) {
    return make_float2(a.x + b.x, a.y + b.y);
}
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

// a*m0 + b*m1 with the products fused into FMAs
__device__ __forceinline__ float2 cmac2(float2 a, float2 m0, float2 b, float2 m1) {
    float re = a.x * m0.x;
    re = fmaf(-a.y, m0.y, re);
    re = fmaf(b.x, m1.x, re);
    re = fmaf(-b.y, m1.y, re);
    float im = a.x * m0.y;
    im = fmaf(a.y, m0.x, im);
    im = fmaf(b.x, m1.y, im);
    im = fmaf(b.y, m1.x, im);
    return make_float2(re, im);
}

// Row-vector 2x2 (out = in @ M on a pair) of a rotation by angle theta, the
// matrix qandle assembles as _a * a_op(t) + _b * b_op(t) with t = theta / 2
// and transposed buffers (qandle/operators.py:236-238, :265-275, :368-395):
//   RX [[c, -is], [-is, c]]   RY [[c, s], [-s, c]]   RZ diag(c - is, c + is)
// m[0]=M00 m[1]=M01 m[2]=M10 m[3]=M11.
__device__ __forceinline__ void rotation_row_matrix(int axis, float theta, float2 m[4]) {
    float s, c;
    sincosf(0.5f * theta, &s, &c);
    if (axis == AX_X) {
        m[0] = make_float2(c, 0.f);
        m[1] = make_float2(0.f, -s);
        m[2] = make_float2(0.f, -s);
        m[3] = make_float2(c, 0.f);
    } else if (axis == AX_Y) {
        m[0] = make_float2(c, 0.f);
        m[1] = make_float2(s, 0.f);
        m[2] = make_float2(-s, 0.f);
        m[3] = make_float2(c, 0.f);
    } else {
        m[0] = make_float2(c, -s);
        m[1] = make_float2(0.f, 0.f);
        m[2] = make_float2(0.f, 0.f);
        m[3] = make_float2(c, s);
    }
}

// Row form of the inverse: in @ M^dagger.
__host__ __device__ __forceinline__ void dagger_row_matrix(float2 m[4]) {
    float2 a = m[0], b = m[1], c = m[2], d = m[3];
    m[0] = cconj(a);
    m[1] = cconj(c);
    m[2] = cconj(b);
    m[3] = cconj(d);
}

// o0 = a0*M00 + a1*M10 ; o1 = a0*M01 + a1*M11
__device__ __forceinline__ void apply_row2(float2& a0, float2& a1, const float2 m[4]) {
    float2 o0 = cmac2(a0, m[0], a1, m[2]);
    float2 o1 = cmac2(a0, m[1], a1, m[3]);
    a0 = o0;
    a1 = o1;
}

// Generator P of a rotation applied (column convention) to the pair (a0, a1):
// dR/dtheta = -i/2 P R.
__device__ __forceinline__ void apply_pauli(int axis, float2& a0, float2& a1) {
    if (axis == AX_X) {
        float2 t = a0;
        a0 = a1;
        a1 = t;
    } else if (axis == AX_Y) {  // Y = [[0, -i], [i, 0]]
        float2 b0 = make_float2(a1.y, -a1.x);
        float2 b1 = make_float2(-a0.y, a0.x);
        a0 = b0;
        a1 = b1;
    } else {
        a1 = make_float2(-a1.x, -a1.y);
    }
}

// Insert a zero bit at position p of x.
__host__ __device__ __forceinline__ uint64_t insert_zero(uint64_t x, int p) {
    uint64_t lo = x & ((uint64_t(1) << p) - 1);
    return ((x >> p) << (p + 1)) | lo;
}

}  // namespace qg

// Plain form: one coalesced, vectorised HBM pass per gate.
//
// These kernels are the per-layer drop-in for the reference's Built*.forward
// modules, which apply every gate as a dense 2^n x 2^n matmul:
//   BuiltRX/RY/RZ.forward   qandle/operators.py:289-298
//   BuiltU.forward          qandle/operators.py:125-126
//   BuiltCNOT/CZ/SWAP       qandle/operators.py:565-566, :597-598, :676-677
//   AngleEmbeddingBuilt     qandle/embeddings.py:148-164
//   MeasureProbabilityBuilt qandle/measurements.py:120-123
//   MeasureAllAbsolute      qandle/measurements.py:78-79
// Here a gate is O(2^n) index arithmetic on the state in place.  Each thread
// moves 16-byte float4 vectors (two complex64 amplitudes) whenever the gate's
// lowest bit is >= 1, so a warp touches 512 contiguous bytes per access.
#include <mutex>

#include "common.cuh"
#include "qandle_gb300.h"

namespace qg {

struct MatSrc {
    int kind;             // AX_X/AX_Y/AX_Z rotation, or 3 = explicit row matrix
    const float* theta;   // rotation angle(s), device
    int64_t stride;       // 0: one angle for all samples, 1: one per sample
    const float2* mat;    // kind 3: row-form 2x2, device
    int dagger;           // apply the inverse
};

__device__ __forceinline__ void load_matrix(const MatSrc& ms, int64_t b, float2 m[4]) {
    if (ms.kind == 3) {
        m[0] = ms.mat[0];
        m[1] = ms.mat[1];
        m[2] = ms.mat[2];
        m[3] = ms.mat[3];
    } else {
        rotation_row_matrix(ms.kind, __ldg(ms.theta + ms.stride * b), m);
    }
    if (ms.dagger) dagger_row_matrix(m);
}

// n >= 2: each thread applies the gate to two pairs held in two float4s.
__global__ void k_1q_vec(float4* __restrict__ s4, int64_t units, int n, int p, MatSrc ms) {
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; u < units; u += (int64_t)gridDim.x * blockDim.x) {
        uint64_t i0, i1;  // amplitude index of the first element of each float4
        if (p == 0) {
            i0 = 4 * (uint64_t)u;
            i1 = i0 + 2;
        } else {
            i0 = insert_zero(2 * (uint64_t)u, p);
            i1 = i0 + (uint64_t(1) << p);
        }
        float2 m[4];
        load_matrix(ms, (int64_t)(i0 >> n), m);
        float4 v0 = s4[i0 >> 1], v1 = s4[i1 >> 1];
        float2 a0 = make_float2(v0.x, v0.y), a1 = make_float2(v0.z, v0.w);
        float2 b0 = make_float2(v1.x, v1.y), b1 = make_float2(v1.z, v1.w);
        if (p == 0) {  // pairs inside each float4
            apply_row2(a0, a1, m);
            apply_row2(b0, b1, m);
        } else {
            apply_row2(a0, b0, m);
            apply_row2(a1, b1, m);
        }
        s4[i0 >> 1] = make_float4(a0.x, a0.y, a1.x, a1.y);
        s4[i1 >> 1] = make_float4(b0.x, b0.y, b1.x, b1.y);
    }
}

// n == 1: one pair (one float4) per sample.
__global__ void k_1q_n1(float4* __restrict__ s4, int64_t batch, MatSrc ms) {
    int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= batch) return;
    float2 m[4];
    load_matrix(ms, b, m);
    float4 v = s4[b];
    float2 a0 = make_float2(v.x, v.y), a1 = make_float2(v.z, v.w);
    apply_row2(a0, a1, m);
    s4[b] = make_float4(a0.x, a0.y, a1.x, a1.y);
}

// Controlled 2x2: the gate on bit p acts on the pairs whose control bit c is
// 1 (a quarter of the amplitudes per pair side); the rest stay.  Mirrors
// BuiltControlled.forward (qandle/operators.py:486-503): the target acts on
// the control=1 subspace, the control=0 rows are kept.
__global__ void k_c1q(float2* __restrict__ s, int64_t units, int n, int p, int c, MatSrc ms) {
    const int lo = p < c ? p : c, hi = p < c ? c : p;
    const uint64_t P = uint64_t(1) << p, C = uint64_t(1) << c;
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; u < units; u += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t i0 = insert_zero(insert_zero((uint64_t)u, lo), hi) | C;
        float2 m[4];
        load_matrix(ms, (int64_t)(i0 >> n), m);
        float2 a0 = s[i0], a1 = s[i0 | P];
        apply_row2(a0, a1, m);
        s[i0] = a0;
        s[i0 | P] = a1;
    }
}

// Reset of bit p (qandle/operators.py:612-623): per pair (qubit 0, qubit 1)
// the |0> amplitude is scaled to carry the pair's norm, the |1> amplitude
// becomes 0: a0 *= |pair| / (|a0| + 1e-7), a1 = 0 (float32 like the
// reference).
__global__ void k_reset(float2* __restrict__ s, int64_t units, int p) {
    const uint64_t P = uint64_t(1) << p;
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; u < units; u += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t i0 = insert_zero((uint64_t)u, p);
        const float2 a0 = s[i0], a1 = s[i0 | P];
        const float nrm = sqrtf(a0.x * a0.x + a0.y * a0.y + a1.x * a1.x + a1.y * a1.y);
        const float n0 = sqrtf(a0.x * a0.x + a0.y * a0.y);
        const float sc = nrm / (n0 + 1e-7f);
        s[i0] = make_float2(a0.x * sc, a0.y * sc);
        s[i0 | P] = make_float2(0.f, 0.f);
    }
}

// Swap amplitude i (bit set_bit = 1, bit other = 0) with i ^ flip.
//   CNOT(c -> t): set = c, other = t, flip = 1<<t
//   SWAP(a, b):   set = a, other = b, flip = (1<<a)|(1<<b)
// lo/hi = the two bits sorted.  Vector form when both bits >= 1.
__global__ void k_swap_vec(float4* __restrict__ s4, int64_t units, int lo, int hi,
                           uint64_t setmask, uint64_t flip) {
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; u < units; u += (int64_t)gridDim.x * blockDim.x) {
        uint64_t i = insert_zero(insert_zero(2 * (uint64_t)u, lo), hi) | setmask;
        uint64_t j = i ^ flip;
        float4 a = s4[i >> 1], b = s4[j >> 1];
        s4[i >> 1] = b;
        s4[j >> 1] = a;
    }
}

__global__ void k_swap_scalar(float2* __restrict__ s, int64_t units, int lo, int hi,
                              uint64_t setmask, uint64_t flip) {
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; u < units; u += (int64_t)gridDim.x * blockDim.x) {
        uint64_t i = insert_zero(insert_zero((uint64_t)u, lo), hi) | setmask;
        uint64_t j = i ^ flip;
        float2 a = s[i], b = s[j];
        s[i] = b;
        s[j] = a;
    }
}

// CNOT with target bit 0: swap the halves of every float4 whose control bit is set.
__global__ void k_cnot_t0(float4* __restrict__ s4, int64_t units, int c) {
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; u < units; u += (int64_t)gridDim.x * blockDim.x) {
        // float4 index f has amplitude index 2f; control bit c >= 1 is bit c-1 of f
        uint64_t f = insert_zero((uint64_t)u, c - 1) | (uint64_t(1) << (c - 1));
        float4 v = s4[f];
        s4[f] = make_float4(v.z, v.w, v.x, v.y);
    }
}

// CZ: negate amplitudes with both bits set.
__global__ void k_cz_vec(float4* __restrict__ s4, int64_t units, int lo, int hi, uint64_t mask) {
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; u < units; u += (int64_t)gridDim.x * blockDim.x) {
        uint64_t i = insert_zero(insert_zero(2 * (uint64_t)u, lo), hi) | mask;
        float4 v = s4[i >> 1];
        s4[i >> 1] = make_float4(-v.x, -v.y, -v.z, -v.w);
    }
}

__global__ void k_cz_scalar(float2* __restrict__ s, int64_t units, int lo, int hi, uint64_t mask) {
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; u < units; u += (int64_t)gridDim.x * blockDim.x) {
        uint64_t i = insert_zero(insert_zero((uint64_t)u, lo), hi) | mask;
        float2 v = s[i];
        s[i] = make_float2(-v.x, -v.y);
    }
}

struct EmbedArgs {
    int nq;          // listed qubits (duplicates allowed, applied in order)
    int axis;
    int8_t qubit[64];
};

// Per-sample, per-qubit factor R_q(x)|0> (column 2-vector); unlisted qubits
// keep |0>.  fac: [batch][n][2] float2.  Rotations listed twice on one qubit
// compose, as the reference's matrix product (embeddings.py:156-164) does.
__global__ void k_embed_factors(float2* __restrict__ fac, const float* __restrict__ x,
                                int64_t xstride, int64_t batch, int n, EmbedArgs ea) {
    int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= batch) return;
    float2* f = fac + b * n * 2;
    for (int q = 0; q < n; ++q) {
        f[2 * q] = make_float2(1.f, 0.f);
        f[2 * q + 1] = make_float2(0.f, 0.f);
    }
    for (int j = 0; j < ea.nq; ++j) {
        int q = ea.qubit[j];
        float2 m[4];
        rotation_row_matrix(ea.axis, x[b * xstride + j], m);
        float2 v0 = f[2 * q], v1 = f[2 * q + 1];
        // column form = transpose of the row form
        f[2 * q] = cmac2(m[0], v0, m[2], v1);
        f[2 * q + 1] = cmac2(m[1], v0, m[3], v1);
    }
}

// out[b][i] = prod_q fac[b][q][bit (n-1-q) of i]; four amplitudes per thread.
__global__ void k_embed_write(float4* __restrict__ out4, const float2* __restrict__ fac,
                              int64_t units, int n) {
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; u < units; u += (int64_t)gridDim.x * blockDim.x) {
        uint64_t i = 4 * (uint64_t)u;
        uint64_t dim = uint64_t(1) << n;
        int64_t b = (int64_t)(i >> n);
        uint64_t k = i & (dim - 1);
        const float2* f = fac + b * n * 2;
        float2 h = make_float2(1.f, 0.f);
        for (int bit = 2; bit < n; ++bit) {
            int q = n - 1 - bit;
            h = cmul(h, f[2 * q + ((k >> bit) & 1)]);
        }
        float2 l[4];
        const float2* f0 = f + 2 * (n - 1);  // qubit n-1 = bit 0
        const float2* f1 = f + 2 * (n - 2);  // qubit n-2 = bit 1
#pragma unroll
        for (int e = 0; e < 4; ++e) l[e] = cmul(cmul(h, f1[(e >> 1) & 1]), f0[e & 1]);
        out4[i >> 1] = make_float4(l[0].x, l[0].y, l[1].x, l[1].y);
        out4[(i >> 1) + 1] = make_float4(l[2].x, l[2].y, l[3].x, l[3].y);
    }
}

__global__ void k_embed_small(float2* __restrict__ out, const float2* __restrict__ fac,
                              int64_t total, int n) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= total) return;
    int64_t b = t >> n;
    uint64_t k = (uint64_t)t & ((uint64_t(1) << n) - 1);
    const float2* f = fac + b * n * 2;
    float2 a = make_float2(1.f, 0.f);
    for (int bit = 0; bit < n; ++bit) a = cmul(a, f[2 * (n - 1 - bit) + ((k >> bit) & 1)]);
    out[t] = a;
}

__global__ void k_probs(const float4* __restrict__ s4, float2* __restrict__ out2, int64_t units) {
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; u < units; u += (int64_t)gridDim.x * blockDim.x) {
        float4 v = s4[u];
        out2[u] = make_float2(v.x * v.x + v.y * v.y, v.z * v.z + v.w * v.w);
    }
}

__global__ void k_probs_scalar(const float2* __restrict__ s, float* __restrict__ out, int64_t count) {
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (u < count) out[u] = s[u].x * s[u].x + s[u].y * s[u].y;
}

// ---- per-sample reductions (deterministic: fixed chunking, fixed order) ----

constexpr int kRedThreads = 256;
constexpr int kChunkBits = 12;  // amplitudes per reduction block: 4096

__device__ __forceinline__ float block_sum(float v, float* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    float r = 0.f;
    if (threadIdx.x < 32) {
        r = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    return r;  // valid in thread 0
}

// AmplitudeEmbedding (qandle/embeddings.py:29-66): the state is the real
// feature vector, padded with pad_value to 2^n entries and optionally
// divided by max(||.||_2, 1e-12) (torch.nn.functional.normalize).
constexpr int kAmpChunkBits = 13;

// partial sums of x^2 over chunks of one sample's features
__global__ void k_amp_partial(const float* __restrict__ x, int64_t stride, int64_t len, int64_t nch,
                              float* __restrict__ part) {
    __shared__ float sh[32];
    const int64_t b = blockIdx.x / nch, ch = blockIdx.x % nch;
    const int64_t lo = ch << kAmpChunkBits;
    int64_t hi = lo + (int64_t(1) << kAmpChunkBits);
    if (hi > len) hi = len;
    float acc = 0.f;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const float v = x[b * stride + i];
        acc += v * v;
    }
    const float r = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
}

// 1 / max(norm, 1e-12) per sample, partials added in fp64 in chunk order
__global__ void k_amp_norm(const float* __restrict__ part, int64_t batch, int64_t nch, double pad_sq,
                           float* __restrict__ inv) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= batch) return;
    double acc = pad_sq;
    for (int64_t c = 0; c < nch; ++c) acc += part[b * nch + c];
    const double nrm = sqrt(acc);
    inv[b] = (float)(1.0 / (nrm > 1e-12 ? nrm : 1e-12));
}

__global__ void k_amp_write(float2* __restrict__ out, const float* __restrict__ x, int64_t stride, int64_t len,
                            int n, int64_t total, float pad, const float* __restrict__ inv) {
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; u < total; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = u >> n, i = u & ((int64_t(1) << n) - 1);
        float v = i < len ? x[b * stride + i] : pad;
        if (inv) v *= inv[b];
        out[u] = make_float2(v, 0.f);
    }
}


// P0 partials: block (chunk, sample) writes, for each bit j < c, the sum of
// |a|^2 over its amplitudes with bit j clear, and the chunk total at slot c.
__global__ void k_p0_partial(const float2* __restrict__ s, float* __restrict__ part, int n, int c) {
    __shared__ float sh[32];
    int64_t nch = (int64_t(1) << n) >> c;
    int64_t b = blockIdx.x / nch;
    int64_t ch = blockIdx.x % nch;
    const float2* base = s + (b << n) + (ch << c);
    float acc[kChunkBits];
    float tot = 0.f;
#pragma unroll
    for (int j = 0; j < kChunkBits; ++j) acc[j] = 0.f;
    for (int i = threadIdx.x; i < (1 << c); i += blockDim.x) {
        float2 a = base[i];
        float p = a.x * a.x + a.y * a.y;
        tot += p;
#pragma unroll
        for (int j = 0; j < kChunkBits; ++j)
            if (j < c && !((i >> j) & 1)) acc[j] += p;
    }
    float* out = part + (b * nch + ch) * (c + 1);
    for (int j = 0; j < c; ++j) {
        float r = block_sum(acc[j], sh);
        if (threadIdx.x == 0) out[j] = r;
    }
    float r = block_sum(tot, sh);
    if (threadIdx.x == 0) out[c] = r;
}

// P0[b][q] = sum over chunks, in double, in chunk order.
__global__ void k_p0_final(const float* __restrict__ part, float* __restrict__ out, int64_t batch,
                           int n, int c, int64_t nch) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= batch * n) return;
    int64_t b = t / n;
    int q = (int)(t % n);
    int j = n - 1 - q;
    double acc = 0.0;
    const float* p = part + b * nch * (c + 1);
    for (int64_t ch = 0; ch < nch; ++ch) {
        if (j < c)
            acc += p[ch * (c + 1) + j];
        else if (!(((uint64_t)ch << c) >> j & 1))
            acc += p[ch * (c + 1) + c];
    }
    out[t] = (float)acc;
}

// Rotation gradient partials: Im(conj(g_i) (P psi)_i) summed over a chunk of
// pairs of one sample.  grad = 0.5 * that sum  (torch's g = 2 dL/dpsi*).
__global__ void k_rotgrad_partial(const float2* __restrict__ psi, const float2* __restrict__ g,
                                  float* __restrict__ part, int n, int p, int axis, int c, uint64_t cmask) {
    __shared__ float sh[32];
    int64_t nch = (int64_t(1) << (n - 1)) >> c;
    int64_t b = blockIdx.x / nch, ch = blockIdx.x % nch;
    uint64_t P = uint64_t(1) << p;
    float acc = 0.f;
    for (int k = threadIdx.x; k < (1 << c); k += blockDim.x) {
        uint64_t pair = ((uint64_t)ch << c) + k;  // pair index within the sample
        uint64_t i0 = insert_zero(pair, p);
        if ((i0 & cmask) != cmask) continue;  // controlled gate: control-0 pairs do not depend on the angle
        uint64_t base = (uint64_t)b << n;
        float2 a0 = psi[base + i0], a1 = psi[base + (i0 | P)];
        float2 g0 = g[base + i0], g1 = g[base + (i0 | P)];
        apply_pauli(axis, a0, a1);
        float2 t0 = cmul(cconj(g0), a0), t1 = cmul(cconj(g1), a1);
        acc += t0.y + t1.y;
    }
    float r = block_sum(acc, sh);
    if (threadIdx.x == 0) part[b * nch + ch] = r;
}

__global__ void k_rotgrad_final(const float* __restrict__ part, float* __restrict__ out,
                                int64_t batch, int64_t nch, int per_sample) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (per_sample) {
        if (t >= batch) return;
        double acc = 0.0;
        for (int64_t ch = 0; ch < nch; ++ch) acc += part[t * nch + ch];
        out[t] = (float)(0.5 * acc);
    } else {
        if (t != 0) return;
        double acc = 0.0;
        for (int64_t i = 0; i < batch * nch; ++i) acc += part[i];
        out[0] = (float)(0.5 * acc);
    }
}

// grad of |psi|^2: out_i = 2 g_i psi_i (torch's complex gradient convention)
__global__ void k_probs_bwd(const float2* __restrict__ s, const float* __restrict__ g,
                            float2* __restrict__ out, int64_t count) {
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; u < count; u += (int64_t)gridDim.x * blockDim.x) {
        float w = 2.f * g[u];
        float2 a = s[u];
        out[u] = make_float2(w * a.x, w * a.y);
    }
}

// grad of P0: out_i = 2 (sum_q g[b][q] [bit (n-1-q) of i clear]) psi_i
__global__ void k_p0_bwd(const float2* __restrict__ s, const float* __restrict__ g,
                         float2* __restrict__ out, int64_t total, int n) {
    int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; u < total; u += (int64_t)gridDim.x * blockDim.x) {
        int64_t b = u >> n;
        uint64_t k = (uint64_t)u & ((uint64_t(1) << n) - 1);
        const float* gb = g + b * n;
        float w = 0.f;
        for (int q = 0; q < n; ++q)
            if (!((k >> (n - 1 - q)) & 1)) w += gb[q];
        w *= 2.f;
        float2 a = s[u];
        out[u] = make_float2(w * a.x, w * a.y);
    }
}

static int check_state(const void* state, int64_t batch, int n) {
    QG_CHECK_ARG(state != nullptr, "state is null");
    QG_CHECK_ARG(batch >= 1, "batch must be >= 1");
    QG_CHECK_ARG(n >= 0 && n <= 34, "num_qubits must be in [0, 34]");
    QG_CHECK_ARG(((uintptr_t)state & 15) == 0, "state must be 16-byte aligned");
    return QG_OK;
}

static int launch_1q(void* state, int64_t batch, int n, int qubit, const MatSrc& ms, cudaStream_t st) {
    int rc = check_state(state, batch, n);
    if (rc) return rc;
    QG_CHECK_ARG(qubit >= 0 && qubit < n, "qubit out of range");
    int p = n - 1 - qubit;
    if (n == 1) {
        k_1q_n1<<<grid_for(batch, 256), 256, 0, st>>>((float4*)state, batch, ms);
    } else {
        int64_t units = (batch << n) / 4;
        k_1q_vec<<<grid_for(units, 256), 256, 0, st>>>((float4*)state, units, n, p, ms);
    }
    QG_LAUNCH_CHECK();
    return QG_OK;
}

static int launch_c1q(void* state, int64_t batch, int n, int control, int qubit, const MatSrc& ms,
                      cudaStream_t st) {
    int rc = check_state(state, batch, n);
    if (rc) return rc;
    QG_CHECK_ARG(n >= 2, "a controlled gate needs two qubits");
    QG_CHECK_ARG(qubit >= 0 && qubit < n && control >= 0 && control < n, "qubit out of range");
    QG_CHECK_ARG(qubit != control, "control and target must differ");
    int64_t units = (batch << n) / 4;
    k_c1q<<<grid_for(units, 256), 256, 0, st>>>((float2*)state, units, n, n - 1 - qubit, n - 1 - control, ms);
    QG_LAUNCH_CHECK();
    return QG_OK;
}

}  // namespace qg

using namespace qg;

extern "C" {

int qg_apply_rotation(void* state, int64_t batch, int n, int qubit, int axis, const float* theta,
                      int64_t theta_stride, int dagger, void* stream) {
    QG_CHECK_ARG(axis >= 0 && axis <= 2, "axis must be 0 (x), 1 (y) or 2 (z)");
    QG_CHECK_ARG(theta != nullptr, "theta is null");
    QG_CHECK_ARG(theta_stride == 0 || theta_stride == 1, "theta_stride must be 0 or 1");
    MatSrc ms{axis, theta, theta_stride, nullptr, dagger};
    return launch_1q(state, batch, n, qubit, ms, (cudaStream_t)stream);
}

int qg_apply_matrix(void* state, int64_t batch, int n, int qubit, const void* row_matrix,
                    int dagger, void* stream) {
    QG_CHECK_ARG(row_matrix != nullptr, "matrix is null");
    MatSrc ms{3, nullptr, 0, (const float2*)row_matrix, dagger};
    return launch_1q(state, batch, n, qubit, ms, (cudaStream_t)stream);
}

int qg_apply_controlled_rotation(void* state, int64_t batch, int n, int control, int qubit, int axis,
                                 const float* theta, int64_t theta_stride, int dagger, void* stream) {
    QG_CHECK_ARG(axis >= 0 && axis <= 2, "axis must be 0 (x), 1 (y) or 2 (z)");
    QG_CHECK_ARG(theta != nullptr, "theta is null");
    QG_CHECK_ARG(theta_stride == 0 || theta_stride == 1, "theta_stride must be 0 or 1");
    MatSrc ms{axis, theta, theta_stride, nullptr, dagger};
    return launch_c1q(state, batch, n, control, qubit, ms, (cudaStream_t)stream);
}

int qg_apply_controlled_matrix(void* state, int64_t batch, int n, int control, int qubit,
                               const void* row_matrix, int dagger, void* stream) {
    QG_CHECK_ARG(row_matrix != nullptr, "matrix is null");
    MatSrc ms{3, nullptr, 0, (const float2*)row_matrix, dagger};
    return launch_c1q(state, batch, n, control, qubit, ms, (cudaStream_t)stream);
}

int64_t qg_amplitude_embedding_scratch_bytes(int64_t batch, int64_t len) {
    const int64_t nch = (len + (int64_t(1) << kAmpChunkBits) - 1) >> kAmpChunkBits;
    return (batch * (nch > 0 ? nch : 1) + batch) * (int64_t)sizeof(float);
}

int qg_amplitude_embedding(void* out, const float* x, int64_t x_row_stride, int64_t batch, int n, int64_t len,
                           float pad_value, int normalize, void* scratch, int64_t scratch_bytes, void* stream) {
    int rc = check_state(out, batch, n);
    if (rc) return rc;
    QG_CHECK_ARG(x != nullptr, "x is null");
    QG_CHECK_ARG(len >= 0 && len <= (int64_t(1) << n), "feature count must be in [0, 2^n]");
    QG_CHECK_ARG(x_row_stride >= len, "x_row_stride must be >= the feature count");
    cudaStream_t st = (cudaStream_t)stream;
    const float* inv = nullptr;
    if (normalize) {
        QG_CHECK_ARG(scratch != nullptr && scratch_bytes >= qg_amplitude_embedding_scratch_bytes(batch, len),
                     "scratch too small");
        const int64_t nch = (len + (int64_t(1) << kAmpChunkBits) - 1) >> kAmpChunkBits;
        float* part = (float*)scratch;
        float* invb = part + batch * (nch > 0 ? nch : 1);
        if (nch > 0) {
            QG_CHECK_ARG(batch * nch < (int64_t(1) << 31), "batch * chunks must be < 2^31");
            k_amp_partial<<<(unsigned)(batch * nch), kRedThreads, 0, st>>>(x, x_row_stride, len, nch, part);
            QG_LAUNCH_CHECK();
        }
        const double pad_sq = (double)pad_value * pad_value * (double)((int64_t(1) << n) - len);
        k_amp_norm<<<grid_for(batch, 128), 128, 0, st>>>(part, batch, nch, pad_sq, invb);
        QG_LAUNCH_CHECK();
        inv = invb;
    }
    const int64_t total = batch << n;
    k_amp_write<<<grid_for(total, 256), 256, 0, st>>>((float2*)out, x, x_row_stride, len, n, total, pad_value, inv);
    QG_LAUNCH_CHECK();
    return QG_OK;
}

int qg_reset(void* state, int64_t batch, int n, int qubit, void* stream) {
    int rc = check_state(state, batch, n);
    if (rc) return rc;
    QG_CHECK_ARG(qubit >= 0 && qubit < n, "qubit out of range");
    int64_t units = (batch << n) / 2;
    cudaStream_t st = (cudaStream_t)stream;
    k_reset<<<grid_for(units, 256), 256, 0, st>>>((float2*)state, units, n - 1 - qubit);
    QG_LAUNCH_CHECK();
    return QG_OK;
}

static int launch_pair_swap(void* state, int64_t batch, int n, int qa, int qb, int is_swap,
                            cudaStream_t st) {
    int rc = check_state(state, batch, n);
    if (rc) return rc;
    QG_CHECK_ARG(qa >= 0 && qa < n && qb >= 0 && qb < n, "qubit out of range");
    QG_CHECK_ARG(qa != qb, "the two qubits must differ");
    int a = n - 1 - qa, b = n - 1 - qb;
    uint64_t A = uint64_t(1) << a, Bm = uint64_t(1) << b;
    int lo = a < b ? a : b, hi = a < b ? b : a;
    uint64_t setmask = A, flip = is_swap ? (A | Bm) : Bm;
    int64_t total = batch << n;
    if (!is_swap && b == 0) {  // CNOT onto bit 0: swap halves of float4s (control >= 1)
        int64_t units = total / 4;
        k_cnot_t0<<<grid_for(units, 256), 256, 0, st>>>((float4*)state, units, a);
    } else if (lo >= 1) {
        int64_t units = total / 8;
        k_swap_vec<<<grid_for(units, 256), 256, 0, st>>>((float4*)state, units, lo, hi, setmask, flip);
    } else {
        int64_t units = total / 4;
        k_swap_scalar<<<grid_for(units, 256), 256, 0, st>>>((float2*)state, units, lo, hi, setmask, flip);
    }
    QG_LAUNCH_CHECK();
    return QG_OK;
}

int qg_apply_cnot(void* state, int64_t batch, int n, int control, int target, void* stream) {
    return launch_pair_swap(state, batch, n, control, target, 0, (cudaStream_t)stream);
}

int qg_apply_swap(void* state, int64_t batch, int n, int qa, int qb, void* stream) {
    return launch_pair_swap(state, batch, n, qa, qb, 1, (cudaStream_t)stream);
}

int qg_apply_cz(void* state, int64_t batch, int n, int control, int target, void* stream) {
    int rc = check_state(state, batch, n);
    if (rc) return rc;
    QG_CHECK_ARG(control >= 0 && control < n && target >= 0 && target < n, "qubit out of range");
    QG_CHECK_ARG(control != target, "control and target must differ");
    int a = n - 1 - control, b = n - 1 - target;
    int lo = a < b ? a : b, hi = a < b ? b : a;
    uint64_t mask = (uint64_t(1) << a) | (uint64_t(1) << b);
    int64_t total = batch << n;
    cudaStream_t st = (cudaStream_t)stream;
    if (lo >= 1) {
        int64_t units = total / 8;
        k_cz_vec<<<grid_for(units, 256), 256, 0, st>>>((float4*)state, units, lo, hi, mask);
    } else {
        int64_t units = total / 4;
        k_cz_scalar<<<grid_for(units, 256), 256, 0, st>>>((float2*)state, units, lo, hi, mask);
    }
    QG_LAUNCH_CHECK();
    return QG_OK;
}

int64_t qg_angle_embedding_scratch_bytes(int64_t batch, int n) {
    return batch * (int64_t)n * 2 * (int64_t)sizeof(float2);
}

int qg_angle_embedding(void* out, const float* x, int64_t x_row_stride, int64_t batch, int n,
                       const int* qubits, int nq, int axis, void* scratch, int64_t scratch_bytes,
                       void* stream) {
    int rc = check_state(out, batch, n);
    if (rc) return rc;
    QG_CHECK_ARG(n >= 1, "AngleEmbedding needs at least one qubit");
    QG_CHECK_ARG(axis >= 0 && axis <= 2, "rotation must be rx, ry or rz");
    QG_CHECK_ARG(nq >= 0 && nq <= 64, "at most 64 embedded angles");
    QG_CHECK_ARG(nq == 0 || (x != nullptr && qubits != nullptr), "x / qubits is null");
    QG_CHECK_ARG(scratch != nullptr && scratch_bytes >= qg_angle_embedding_scratch_bytes(batch, n),
                 "scratch too small");
    EmbedArgs ea;
    ea.nq = nq;
    ea.axis = axis;
    for (int j = 0; j < nq; ++j) {
        QG_CHECK_ARG(qubits[j] >= 0 && qubits[j] < n, "embedded qubit out of range");
        ea.qubit[j] = (int8_t)qubits[j];
    }
    cudaStream_t st = (cudaStream_t)stream;
    float2* fac = (float2*)scratch;
    k_embed_factors<<<grid_for(batch, 128), 128, 0, st>>>(fac, x, x_row_stride, batch, n, ea);
    QG_LAUNCH_CHECK();
    int64_t total = batch << n;
    if (n >= 2) {
        int64_t units = total / 4;
        k_embed_write<<<grid_for(units, 256), 256, 0, st>>>((float4*)out, fac, units, n);
    } else {
        k_embed_small<<<grid_for(total, 256), 256, 0, st>>>((float2*)out, fac, total, n);
    }
    QG_LAUNCH_CHECK();
    return QG_OK;
}

int qg_probs(const void* state, float* out, int64_t count, void* stream) {
    QG_CHECK_ARG(state != nullptr && out != nullptr, "null pointer");
    QG_CHECK_ARG(count >= 0, "count must be >= 0");
    if (count == 0) return QG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (count % 2 == 0 && ((uintptr_t)state & 15) == 0 && ((uintptr_t)out & 7) == 0) {
        int64_t units = count / 2;
        k_probs<<<grid_for(units, 256), 256, 0, st>>>((const float4*)state, (float2*)out, units);
    } else {
        k_probs_scalar<<<grid_for(count, 256), 256, 0, st>>>((const float2*)state, out, count);
    }
    QG_LAUNCH_CHECK();
    return QG_OK;
}

int qg_probs_backward(const void* state, const float* grad_probs, void* grad_state, int64_t count,
                      void* stream) {
    QG_CHECK_ARG(state != nullptr && grad_probs != nullptr && grad_state != nullptr, "null pointer");
    if (count <= 0) return QG_OK;
    k_probs_bwd<<<grid_for(count, 256), 256, 0, (cudaStream_t)stream>>>(
        (const float2*)state, grad_probs, (float2*)grad_state, count);
    QG_LAUNCH_CHECK();
    return QG_OK;
}

int qg_measure_p0_backward(const void* state, const float* grad_p0, void* grad_state, int64_t batch,
                           int n, void* stream) {
    int rc = check_state(state, batch, n);
    if (rc) return rc;
    QG_CHECK_ARG(grad_p0 != nullptr && grad_state != nullptr, "null pointer");
    int64_t total = batch << n;
    k_p0_bwd<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>(
        (const float2*)state, grad_p0, (float2*)grad_state, total, n);
    QG_LAUNCH_CHECK();
    return QG_OK;
}

int64_t qg_measure_p0_scratch_bytes(int64_t batch, int n) {
    int c = n < kChunkBits ? n : kChunkBits;
    int64_t nch = (int64_t(1) << n) >> c;
    return batch * nch * (c + 1) * (int64_t)sizeof(float);
}

int qg_measure_p0(const void* state, float* out, int64_t batch, int n, void* scratch,
                  int64_t scratch_bytes, void* stream) {
    int rc = check_state(state, batch, n);
    if (rc) return rc;
    QG_CHECK_ARG(out != nullptr, "out is null");
    QG_CHECK_ARG(batch * (((int64_t(1) << n) >> (n < kChunkBits ? n : kChunkBits))) < (int64_t(1) << 31),
                 "batch * chunks must be < 2^31");
    QG_CHECK_ARG(scratch != nullptr && scratch_bytes >= qg_measure_p0_scratch_bytes(batch, n),
                 "scratch too small");
    if (n == 0) return QG_OK;
    int c = n < kChunkBits ? n : kChunkBits;
    int64_t nch = (int64_t(1) << n) >> c;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned grid = (unsigned)(nch * batch);
    k_p0_partial<<<grid, kRedThreads, 0, st>>>((const float2*)state, (float*)scratch, n, c);
    QG_LAUNCH_CHECK();
    k_p0_final<<<grid_for(batch * n, 128), 128, 0, st>>>((const float*)scratch, out, batch, n, c, nch);
    QG_LAUNCH_CHECK();
    return QG_OK;
}

int64_t qg_rotation_grad_scratch_bytes(int64_t batch, int n) {
    int pairs_bits = n - 1;
    int c = pairs_bits < kChunkBits ? pairs_bits : kChunkBits;
    int64_t nch = (int64_t(1) << pairs_bits) >> c;
    return batch * nch * (int64_t)sizeof(float);
}

static int rotation_grad(const void* out_state, const void* grad_out, float* dtheta, int64_t batch, int n,
                         int qubit, int axis, int per_sample, uint64_t cmask, void* scratch,
                         int64_t scratch_bytes, void* stream);

int qg_rotation_grad(const void* out_state, const void* grad_out, float* dtheta, int64_t batch,
                     int n, int qubit, int axis, int per_sample, void* scratch,
                     int64_t scratch_bytes, void* stream) {
    return rotation_grad(out_state, grad_out, dtheta, batch, n, qubit, axis, per_sample, 0, scratch,
                         scratch_bytes, stream);
}

int qg_controlled_rotation_grad(const void* out_state, const void* grad_out, float* dtheta, int64_t batch,
                                int n, int control, int qubit, int axis, int per_sample, void* scratch,
                                int64_t scratch_bytes, void* stream) {
    QG_CHECK_ARG(control >= 0 && control < n && control != qubit, "bad control qubit");
    return rotation_grad(out_state, grad_out, dtheta, batch, n, qubit, axis, per_sample,
                         uint64_t(1) << (n - 1 - control), scratch, scratch_bytes, stream);
}

static int rotation_grad(const void* out_state, const void* grad_out, float* dtheta, int64_t batch, int n,
                         int qubit, int axis, int per_sample, uint64_t cmask, void* scratch,
                         int64_t scratch_bytes, void* stream) {
    int rc = check_state(out_state, batch, n);
    if (rc) return rc;
    QG_CHECK_ARG(grad_out != nullptr && dtheta != nullptr, "null pointer");
    QG_CHECK_ARG(qubit >= 0 && qubit < n, "qubit out of range");
    QG_CHECK_ARG(axis >= 0 && axis <= 2, "axis must be 0..2");
    QG_CHECK_ARG(n >= 1, "no qubits");
    QG_CHECK_ARG(scratch != nullptr && scratch_bytes >= qg_rotation_grad_scratch_bytes(batch, n),
                 "scratch too small");
    int pairs_bits = n - 1;
    int c = pairs_bits < kChunkBits ? pairs_bits : kChunkBits;
    int64_t nch = (int64_t(1) << pairs_bits) >> c;
    cudaStream_t st = (cudaStream_t)stream;
    QG_CHECK_ARG(batch * nch < (int64_t(1) << 31), "batch * chunks must be < 2^31");
    unsigned grid = (unsigned)(nch * batch);
    k_rotgrad_partial<<<grid, kRedThreads, 0, st>>>((const float2*)out_state, (const float2*)grad_out,
                                                   (float*)scratch, n, n - 1 - qubit, axis, c, cmask);
    QG_LAUNCH_CHECK();
    k_rotgrad_final<<<grid_for(per_sample ? batch : 1, 128), 128, 0, st>>>(
        (const float*)scratch, dtheta, batch, nch, per_sample);
    QG_LAUNCH_CHECK();
    return QG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------
// P0 without caller-provided scratch.
//
// Some callers of this library cannot allocate device memory at the point
// where they measure: code running inside a captured or replayed CUDA graph
// that must not add allocation nodes, real-time loops that forbid
// cudaMalloc/cudaFree stalls, and bindings from hosts whose allocator owns
// all device memory and hands out no scratch.  For them the per-chunk
// partial sums live in one fixed array that every device loading this
// library holds until the process exits.
//
// - Limit: QG_P0_NOALLOC_MAX_PARTIALS floats (4 MiB).  A call needs
//   batch * (2^n / 2^min(n, 12)) * (min(n, 12) + 1) of them and is refused
//   beyond that.
// - Set-up: the first call on a device looks up the array's device address
//   (cudaGetSymbolAddress, with that device current) and caches it; make that
//   first call before any stream capture.  A cudaDeviceReset invalidates the
//   cached address; the entry point must not be used on that device again.
// - Sharing: every call uses the same array.  Nothing in it needs to start at
//   zero (each block writes all its partials before the reduction reads
//   them), but calls whose kernels overlap on the GPU (different streams,
//   threads or graphs without ordering) race on it.
static __device__ __align__(256) float g_p0_partials[QG_P0_NOALLOC_MAX_PARTIALS];

namespace {
std::mutex g_p0_partials_mu;
float* g_p0_partials_ptr[256];  // per device ordinal, looked up once
}  // namespace

extern "C" int qg_measure_p0_noalloc(const void* state, float* out, int64_t batch, int n, void* stream) {
    int rc = check_state(state, batch, n);
    if (rc) return rc;
    QG_CHECK_ARG(out != nullptr, "out is null");
    if (n == 0) return QG_OK;
    int c = n < kChunkBits ? n : kChunkBits;
    int64_t nch = (int64_t(1) << n) >> c;
    // per-sample need first, so that a huge batch cannot wrap the product
    const int64_t per_sample = nch * (c + 1);
    if (batch > (int64_t)QG_P0_NOALLOC_MAX_PARTIALS / per_sample) {
        qg::set_error("qg_measure_p0_noalloc: batch " + std::to_string(batch) + " at " + std::to_string(n) +
                      " qubits needs " + std::to_string(per_sample) +
                      " partial sums per sample, more than the static array holds (" +
                      std::to_string((int64_t)QG_P0_NOALLOC_MAX_PARTIALS) +
                      "); use qg_measure_p0 with a caller-provided scratch buffer");
        return QG_ENOMEM;
    }
    int dev = 0;
    QG_CUDA_TRY(cudaGetDevice(&dev));
    QG_CHECK_ARG(dev >= 0 && dev < 256, "device ordinal out of range");
    float* part = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_p0_partials_mu);
        if (!g_p0_partials_ptr[dev]) {
            void* p = nullptr;
            QG_CUDA_TRY(cudaGetSymbolAddress(&p, g_p0_partials));
            g_p0_partials_ptr[dev] = (float*)p;
        }
        part = g_p0_partials_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    unsigned grid = (unsigned)(nch * batch);
    k_p0_partial<<<grid, kRedThreads, 0, st>>>((const float2*)state, part, n, c);
    QG_LAUNCH_CHECK();
    k_p0_final<<<grid_for(batch * n, 128), 128, 0, st>>>(part, out, batch, n, c, nch);
    QG_LAUNCH_CHECK();
    return QG_OK;
}

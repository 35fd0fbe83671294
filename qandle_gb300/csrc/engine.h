// Internal descriptors shared by the fusion planner (program.cpp) and the
// fused pass kernels (fused.cu).  All structs are plain data copied verbatim
// to device memory.
#pragma once
#ifndef __CUDACC_RTC__
#include <stdint.h>
#endif

namespace qg {

constexpr int kRegBits = 5;         // amplitudes per thread = 2^5, held in registers
constexpr int kMaxTileBits = 13;    // forward tile: 2^13 amplitudes, 256 threads, 64 KiB
constexpr int kMaxQubits = 30;      // fused engine limit (global bit masks are 32-bit)
// register bits of the backward pass kernel (psi and lambda tiles per thread)
constexpr int kBwdRegBits = 4;
// backward: gradient slots per pass (their partials live in shared memory
// beside the psi/lambda double buffer, 5 B per slot and thread)
__host__ __device__ constexpr int max_grad_per_pass(int reg_bits) { return reg_bits == 4 ? 64 : 96; }

// Tile buffers of the forward kernel: three (the compute warps work on tile
// t while the producer warp stores tile t-2 out of the third buffer and then
// loads tile t+1 into it).  Two 2^12 CTAs with three buffers each still fit
// one SM's shared memory.
__host__ __device__ constexpr int fwd_stages(int) { return 3; }

// Producer warps of a forward CTA: they move the tiles between global and
// shared memory, each warp a fixed share of every tile's rows.
__host__ __device__ constexpr int fwd_producer_warps(int tb) { return tb >= 13 ? 4 : 2; }

// Threads of a forward CTA: 2^(TB-RB) compute threads (2^RB amplitudes each)
// and the producer warps.
__host__ __device__ constexpr int fwd_threads(int tb, int rb) {
    return (1 << (tb - rb)) + 32 * fwd_producer_warps(tb);
}

// Resident CTAs per SM the launch bounds ask for.  The compiler caps a thread
// at 65536 / (threads x CTAs) registers: 168 for the compute threads of
// RB = 5 (32 amplitudes), about 100 for RB = 4.
__host__ __device__ constexpr int fwd_min_blocks(int tb, int rb) {
    return tb >= 13 ? 1 : tb == 12 ? 2 : 3;
}

// Shared-memory swizzle of the exchanges.  The exchange planes hold 2^TB
// floats; local index j goes to slot j ^ L(j >> 5), where L XORs into the low
// five bits (the 4-byte bank) the image swz_image(k) of every set high bit
// 5 + k.  Local bit b < 5 has image 1 << b.  A warp's exchange access is free
// of bank conflicts when its five lane bits have independent images; the
// images below leave independent lane choices after taking out the register
// bits for all but 3 of the 1287 register sets of a 2^13 tile with 5
// register bits (1 of 495 at 2^12 with 4), where bank = (b mod 5) left 450.
__host__ __device__ constexpr int swz_image(int k) {
    return k == 0 ? 14 : k == 1 ? 25 : k == 2 ? 7 : k == 3 ? 26 : k == 4 ? 19 : k == 5 ? 31 : k == 6 ? 22 : 11;
}
// Bank image of local bit b (the low five bits of its slot offset).
__host__ __device__ constexpr int bank_image(int b) { return b < 5 ? (1 << b) : swz_image(b - 5); }
__host__ __device__ constexpr int swz_slot(int j) {
    int h = j >> 5, x = 0;
    for (int k = 0; k < 8; ++k)
        if ((h >> k) & 1) x ^= swz_image(k);
    return j ^ x;
}

// Device op codes (int4 per op: x = opcode, y/z/w operands).
enum Opcode : int32_t {
    OP_MAP = 1,   // exchange through shared memory to a new register/lane/warp mapping
                  //   y = 5 register local bits (4 bits each), z = 5 lane local bits,
                  //   w = warp local bits (4 bits each) | (count << 16)
    OP_MAT = 2,   // 2x2 on register position y with matrix slot z; w = flags
    OP_DIAG = 3,  // diag(m00, m11) on the bit at location y with slot z; w = flags
    OP_CX = 4,    // X on register position y when the control at location z is 1
    OP_CZ = 5,    // negate when the bits at locations y and z are both 1
    OP_SWAP = 6,  // exchange register positions y and z
    OP_GRAD = 7,  // backward: gradient partial Im<lam|P|psi> of axis z on register
                  //   position y into grad slot w (no state change)
    OP_XMAT = 8,  // apply the pending X of register position y to the registers
                  //   (no state change: inserted before an exchange whose writes
                  //   it would bank-conflict)
};
constexpr int32_t LOC_REG = 0x100;  // location = register position (low bits); else global bit
constexpr int32_t OPF_PER_SAMPLE = 1;  // matrix slot is per sample
constexpr int32_t OPF_GRAD = 2;        // OP_MAT in the backward: gradient first (axis in bits 8..9)

enum InitKind : int32_t { INIT_LOAD = 0, INIT_ZERO = 1, INIT_EMBED = 2 };
enum EpiFlags : int32_t { EPI_STORE = 1, EPI_PROBS = 2, EPI_P0 = 4 };

struct PassDesc {
    int32_t tile_bits;        // TB (13 forward, 12 backward)
    int32_t nq_tile;          // local bits that are qubits: min(n, TB); the rest are sample bits
    int32_t run_bits;         // low local bits contiguous in memory
    int32_t nfixed;           // qubit bits outside the tile (n - nq_tile)
    int32_t gbit[16];         // local bit -> global bit (local < nq_tile)
    int32_t fixed_gbit[32];   // global bits outside the tile, ascending
    int32_t op_begin, op_count;
    int32_t init;             // InitKind
    int32_t epi;              // EpiFlags
    int32_t init_map[3];      // mapping the init produces (OP_MAP encoding y, z, w)
    int32_t ckpt;             // forward: also store the state into checkpoint ckpt (-1: none)
    int32_t grad_base;        // backward: first grad slot of this pass
    int32_t ngrad;            // backward: grad slots in this pass
    int32_t psi_from_ckpt;    // backward: read psi from checkpoint (>= 0) instead of the state
    int32_t end_map[3];       // mapping the gate program ends in (OP_MAP encoding); its lanes
                              // are local bits 0..4, so the tile is written back from it
};

struct SlotDesc {
    int32_t chain_begin, chain_len;
    int32_t per_sample;       // 1: one matrix per sample
    int32_t out_index;        // index within the shared or per-sample matrix table
};

struct ChainEntry {
    int32_t kind;    // 0..2 rotation axis, 3 = explicit row matrix
    int32_t src;     // rotation: 0 = params[idx], 1 = named[b][idx]; matrix: umats[idx]
    int32_t idx;
    int32_t dagger;  // use the inverse
};

struct GradTarget {
    int32_t src;     // 0 = params[idx] (summed over samples), 1 = named[b][idx]
    int32_t idx;
};

struct EmbedDesc {
    int32_t axis;
    int32_t nq;
    int32_t col0;        // first named column
    int32_t pad;
    int8_t qubit[64];
};

// Launch-time pointers of one fused program run (forward or backward).
struct RunArgs {
    float2* state;            // [B][2^n] working state (psi)
    float2* lam;              // backward: cotangent [B][2^n]
    float2* ckpt;             // checkpoints [nckpt][B][2^n] (may be null)
    float* out;               // probs [B][2^n] (EPI_PROBS)
    float* p0part;            // P0 partials [B][tps][TB + 1] (EPI_P0)
    float* gradpart;          // backward: grad partials [grad slot][tiles]
    const float2* mats;       // shared matrices [S][4]
    const float2* mats_ps;    // per-sample matrices [B][P][4]
    const float2* embfac;     // embedding factors [B][n][2]
    int* status;              // device status word (bounded waits)
    int64_t batch;
    int32_t n;
    int32_t nslots_ps;        // P
    int32_t nslots_shared;    // S
    int32_t pad_;
};

// Shared-memory copies the pass kernels keep of the current pass's op list
// and of the shared matrix table (longer lists / tables stay in global memory).
constexpr int kSmemOps = 512;
constexpr int kSmemMats = 256;
// Compiled forward passes keep no op list; the op-list area holds the
// per-sample matrices of the tile in each of the three buffers instead, up to
// this many 2x2 matrices (32 bytes) per buffer.
constexpr int kStagedPerSlot = kSmemOps * 16 / 3 / 32;

// Dynamic shared memory of the forward kernel: the tile ring, the op list,
// the shared matrix table and the full/empty mbarrier of each tile buffer.
__host__ __device__ constexpr int fwd_smem_bytes(int tb) {
    return fwd_stages(tb) * (1 << tb) * 8 + kSmemOps * 16 + kSmemMats * 32 + 2 * fwd_stages(tb) * 8;
}

// Threads of a backward CTA: 2^(TB-RB) compute threads and one producer warp
// (the backward's compute threads need up to ~224 registers, so there is no
// room for more producer warps).
__host__ __device__ constexpr int bwd_threads(int tb, int rb) { return (1 << (tb - rb)) + 32; }

// Dynamic shared memory of the backward kernel: psi and lambda in two tile
// slots, the op list, the shared matrix table, the gradient partials and
// their sample tags, and the full/empty mbarrier of each slot.
__host__ __device__ constexpr int bwd_smem_bytes(int tb, int rb) {
    return 4 * (1 << tb) * 8 + kSmemOps * 16 + kSmemMats * 32 + max_grad_per_pass(rb) * (1 << (tb - rb)) * 5 +
           4 * 8;
}

#ifndef __CUDACC_RTC__
// Host view of a planned program, for the launch code in fused.cu.
struct ProgramRun {
    int n, tile_bits, reg_bits, measure, keep_state, segments;
    int nparams, ncols, numats, ngrads, has_embed;
    int nfslots, f_shared, f_ps, nbslots, b_shared, b_ps;
    int nfpass, nbpass;
    const PassDesc* fpass;  // host copies
    const PassDesc* bpass;
    const int32_t* fops;    // host op lists (int4 per op)
    const int32_t* bops;
    size_t off_fpass, off_fops, off_fslot, off_fchain;
    size_t off_bpass, off_bops, off_bslot, off_bchain, off_embed, off_pcsr, off_ccsr;
};
void program_run_info(const void* prog, ProgramRun* out);
#endif


}  // namespace qg

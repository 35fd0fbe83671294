// Run-time compiled forward pass kernels.
//
// The op interpreter of the prebuilt forward kernel decodes every op of a
// pass at run time: a register position becomes a switch, a CNOT between two
// register qubits becomes register moves, and the code of every op variant
// competes for the instruction cache.  For one program the op lists are
// fixed, so this file writes each forward pass out as CUDA source -- the
// shared kernel body of fwd_kernel.cuh with the pass's ops unrolled as calls
// to jit_ops.cuh with compile-time register positions -- and compiles it for
// sm_103a with NVRTC.  Matrices, angles and states stay run-time data, so one
// compiled program serves every call with any batch and any parameters.
//
// NVRTC is opened with dlopen: without it qg_program_compile reports an
// error and forward passes keep running on the prebuilt interpreter.  Module
// loading and launches go through driver entry points obtained from the CUDA
// runtime (no link-time libcuda dependency).  Compiled modules are cached
// process-wide by (device, source text), so rebuilding an identical program
// compiles nothing; QG_JIT_CACHE_DIR adds a cache of cubins on disk.
#include <cuda.h>
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <sys/resource.h>
#include <sys/syscall.h>
#include <unistd.h>
#include <nvrtc.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "engine.h"
#include "jit.h"
#include "qandle_gb300.h"

namespace qg {

void program_run_info(const void* prog, ProgramRun* r);
void* program_jit_state(const void* prog);
void program_set_jit_state(void* prog, void* state);

// headers handed to NVRTC (generated from csrc/ by build.py)
extern const int kJitHeaderCount;
extern const char* const kJitHeaderNames[];
extern const char* const kJitHeaderTexts[];

namespace {

// ------------------------------------------------------------ NVRTC --

struct Nvrtc {
    decltype(&nvrtcCreateProgram) create = nullptr;
    decltype(&nvrtcCompileProgram) compile = nullptr;
    decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
    decltype(&nvrtcGetProgramLog) log = nullptr;
    decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
    decltype(&nvrtcGetCUBIN) cubin = nullptr;
    decltype(&nvrtcDestroyProgram) destroy = nullptr;
    decltype(&nvrtcGetErrorString) error_string = nullptr;
    decltype(&nvrtcVersion) version = nullptr;
    std::string why;  // empty when loaded
};

#ifndef QG_CUDA_LIB_DIR
#define QG_CUDA_LIB_DIR "/usr/local/cuda/lib64"
#endif

const Nvrtc& nvrtc() {
    static Nvrtc N;
    static std::once_flag once;
    std::call_once(once, [] {
        const char* names[] = {"libnvrtc.so.13", QG_CUDA_LIB_DIR "/libnvrtc.so.13", "libnvrtc.so",
                               QG_CUDA_LIB_DIR "/libnvrtc.so"};
        void* h = nullptr;
        for (const char* nm : names)
            if ((h = dlopen(nm, RTLD_NOW | RTLD_LOCAL))) break;
        if (!h) {
            N.why = "libnvrtc.so.13 not found";
            return;
        }
#define QG_SYM(field, name)                                          \
    N.field = reinterpret_cast<decltype(N.field)>(dlsym(h, #name)); \
    if (!N.field) {                                                  \
        N.why = "libnvrtc lacks " #name;                             \
        return;                                                      \
    }
        QG_SYM(create, nvrtcCreateProgram)
        QG_SYM(compile, nvrtcCompileProgram)
        QG_SYM(log_size, nvrtcGetProgramLogSize)
        QG_SYM(log, nvrtcGetProgramLog)
        QG_SYM(cubin_size, nvrtcGetCUBINSize)
        QG_SYM(cubin, nvrtcGetCUBIN)
        QG_SYM(destroy, nvrtcDestroyProgram)
        QG_SYM(error_string, nvrtcGetErrorString)
        QG_SYM(version, nvrtcVersion)
#undef QG_SYM
    });
    return N;
}

// ----------------------------------------------------------- driver --

struct Driver {
    decltype(&cuModuleLoadData) load = nullptr;
    decltype(&cuModuleGetFunction) get_function = nullptr;
    decltype(&cuFuncSetAttribute) set_attribute = nullptr;
    decltype(&cuLaunchKernel) launch = nullptr;
    decltype(&cuOccupancyMaxActiveBlocksPerMultiprocessor) occupancy = nullptr;
    decltype(&cuGetErrorString) error_string = nullptr;
    std::string why;
};

const Driver& driver() {
    static Driver D;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFree(nullptr);  // the runtime's primary context is current from here on
#define QG_DRV(field, name)                                                                     \
    {                                                                                           \
        void* fp = nullptr;                                                                     \
        cudaDriverEntryPointQueryResult q{};                                                    \
        if (cudaGetDriverEntryPointByVersion(#name, &fp, 12000, cudaEnableDefault, &q) !=       \
                cudaSuccess ||                                                                  \
            !fp) {                                                                              \
            D.why = "driver entry point " #name " unavailable";                               \
            return;                                                                             \
        }                                                                                       \
        D.field = reinterpret_cast<decltype(D.field)>(fp);                                      \
    }
        QG_DRV(load, cuModuleLoadData)
        QG_DRV(get_function, cuModuleGetFunction)
        QG_DRV(set_attribute, cuFuncSetAttribute)
        QG_DRV(launch, cuLaunchKernel)
        QG_DRV(occupancy, cuOccupancyMaxActiveBlocksPerMultiprocessor)
        QG_DRV(error_string, cuGetErrorString)
#undef QG_DRV
    });
    return D;
}

std::string cu_error(CUresult r) {
    const char* s = nullptr;
    if (driver().error_string) driver().error_string(r, &s);
    return s ? std::string(s) : ("CUresult " + std::to_string((int)r));
}

// ------------------------------------------------------ code writer --

std::string loc_bit(int32_t loc) { return "loc_bit_thread(" + std::to_string(loc) + ", tm.tglob)"; }

// ------------------------------------------------ exchange writer --

// A register/lane/warp mapping in OP_MAP encoding, decoded on the host.
struct MapBits {
    int regl[5] = {0, 0, 0, 0, 0};  // register bit k -> local bit
    int thr[16] = {0};              // thread bit k (lanes, then warps) -> local bit
    int nthr = 0;
};

MapBits decode_mapping(int32_t y, int32_t z, int32_t w, int rb) {
    MapBits m;
    for (int k = 0; k < rb; ++k) m.regl[k] = (y >> (4 * k)) & 15;
    const int nw = (w >> 16) & 7;
    m.nthr = 5 + nw;
    for (int k = 0; k < m.nthr; ++k) m.thr[k] = k < 5 ? ((z >> (4 * k)) & 15) : ((w >> (4 * (k - 5))) & 15);
    return m;
}

// The natural mapping (lanes = local bits 0..4, registers = 5.., warps above).
void natural_mapping(int tb, int rb, int32_t& y, int32_t& z, int32_t& w) {
    y = 0;
    for (int k = 0; k < rb; ++k) y |= (5 + k) << (4 * k);
    z = 0x43210;
    w = 0;
    for (int k = 0; k < tb - 5 - rb; ++k) w |= (5 + rb + k) << (4 * k);
    w |= (tb - 5 - rb) << 16;
}

int swz_host(int j) { return swz_slot(j); }

// "C0, C1, C2, C3, C4": slot offsets of the register bits under a mapping.
std::string reg_offsets(const MapBits& m, int rb) {
    std::string out;
    for (int k = 0; k < 5; ++k) {
        if (k) out += ", ";
        out += std::to_string(k < rb ? swz_host(1 << m.regl[k]) : 0);
    }
    return out;
}

// Statements that set the thread-dependent parts of a mapping: the slot base
// `swb`, the global bits of the thread's qubit bits (tm.tglob) and its sample
// offset in the tile (tm.sample_off) -- what decode_map computes at run time.
std::string thread_part(const MapBits& m, const PassDesc& d) {
    std::string swb = "0", tg = "fixed_val", so = "0";
    for (int k = 0; k < m.nthr; ++k) {
        const int lb = m.thr[k];
        const std::string bit = "tbit(tid, " + std::to_string(k) + ")";
        swb += " ^ (" + bit + " ? " + std::to_string(swz_host(1 << lb)) + " : 0)";
        if (lb < d.nq_tile)
            tg += " | ((uint32_t)" + bit + " << " + std::to_string(d.gbit[lb]) + ")";
        else
            so += " | (" + bit + " << " + std::to_string(lb - d.nq_tile) + ")";
    }
    return "swb = " + swb + "; tm.tglob = " + tg + "; tm.sample_off = " + so + ";";
}

// One exchange from mapping `cur` to (y, z, w); `two` = psi and lambda.
std::string exchange_code(const PassDesc& d, const MapBits& cur, int32_t y, int32_t z, int32_t w, int rb,
                          bool two) {
    const MapBits nxt = decode_mapping(y, z, w, rb);
    const std::string cc = reg_offsets(cur, rb), cn = reg_offsets(nxt, rb);
    std::ostringstream s;
    s << "{ cta_sync<(1 << (TB - RB))>(); const int wb_ = swb ^ xm_xor<" << cc << ">(xm); ";
    if (two)
        s << "cxwrite<TB, RB, " << cc << ">(pp, pt, wb_); cxwrite<TB, RB, " << cc << ">(lp, lt, wb_); ";
    else
        s << "cxwrite<TB, RB, " << cc << ">(plane, pt, wb_); ";
    s << "xm = 0; cta_sync<(1 << (TB - RB))>(); " << thread_part(nxt, d) << " ";
    if (two)
        s << "cxread<TB, RB, " << cn << ">(pp, pt, swb); cxread<TB, RB, " << cn << ">(lp, lt, swb); }\n";
    else
        s << "cxread<TB, RB, " << cn << ">(plane, pt, swb); }\n";
    return s.str();
}

// One forward pass as CUDA source: the shared kernel body with the pass's
// gate program unrolled.
std::string pass_source(const ProgramRun& R, int p) {
    const PassDesc& d = R.fpass[p];
    const int tb = d.tile_bits, rb = R.reg_bits;  // the launch uses the same pair
    const int nt = 1 << (tb - rb);
    const int32_t* ops = R.fops + 4 * (size_t)d.op_begin;
    // With n >= TB a tile lies in one sample, so the pass's per-sample
    // matrices are the same for the whole CTA: the producer warps copy them
    // into shared memory with the tile (the op-list area, unused here, has a
    // share per tile buffer) instead of every thread reading them from global
    // memory at every op.
    std::vector<int32_t> staged;  // per-sample slot of each staged matrix
    std::map<int32_t, int> staged_index;
    if (R.n >= tb) {
        for (int o = 0; o < d.op_count; ++o) {
            const int32_t k = ops[4 * o], z = ops[4 * o + 2], w = ops[4 * o + 3];
            if ((k == OP_MAT || k == OP_DIAG) && (w & OPF_PER_SAMPLE) && !staged_index.count(z)) {
                staged_index[z] = (int)staged.size();
                staged.push_back(z);
            }
        }
        const int cap = kStagedPerSlot;  // the op-list area's share of one tile buffer
        if ((int)staged.size() > cap) {
            staged.clear();
            staged_index.clear();
        }
    }
    int32_t ny, nz, nw;
    natural_mapping(tb, rb, ny, nz, nw);
    const int end_natural = (d.end_map[0] == ny && d.end_map[2] == nw) ? 1 : 0;
    std::ostringstream s;
    s << "#include \"jit_ops.cuh\"\n"
         "namespace qg {\n"
         "struct PassOps {\n"
         "  static constexpr bool kStageOps = false;\n"
      << "  static constexpr int kInit = " << d.init << ";\n"
      << "  static constexpr int kEpi = " << d.epi << ";\n"
      << "  static constexpr int kEndNatural = " << end_natural << ";\n"
      << "  static constexpr uint32_t kStagedBytes = " << 32 * staged.size() << ";\n"
         "  __device__ __forceinline__ static void stage(const RunArgs& A, const TileGeo& g, float4* sm, "
         "uint64_t* bar, int lane) {\n";
    // (called by the 32 lanes of the first producer warp, after its lane 0
    // added kStagedBytes to the buffer's full barrier)
    if (!staged.empty()) {
        s << "    for (int k = lane; k < " << staged.size() << "; k += 32) {\n"
          << "      const int slot = ";
        for (size_t i = 0; i + 1 < staged.size(); ++i) s << "k == " << i << " ? " << staged[i] << " : ";
        s << staged.back() << ";\n"
          << "      bulk_g2s(sm + 2 * k, A.mats_ps + (g.sample * A.nslots_ps + slot) * 4, 32u, bar);\n    }\n";
    }
    s << "  }\n"
         "  template <int TB, int RB>\n"
         "  __device__ __forceinline__ static void apply(PTile<RB>& pt, uint32_t& xm, ThreadMap& tm, "
         "const PassDesc& d, const RunArgs& A, const int4*, const int4* s_ops, const float4* s_mats, float* plane, "
         "int64_t sample0, uint32_t fixed_val, int tid) {\n"
         "    const float4* staged = reinterpret_cast<const float4*>(s_ops);\n"
         "    (void)staged;\n"
         "    int swb = tm.sw_base;\n"
         "    (void)swb;\n";
    MapBits cur;
    {
        int32_t y0, z0, w0;
        natural_mapping(tb, rb, y0, z0, w0);
        if (d.init == INIT_EMBED) y0 = d.init_map[0], z0 = d.init_map[1], w0 = d.init_map[2];
        cur = decode_mapping(y0, z0, w0, rb);
    }
    for (int o = 0; o < d.op_count; ++o) {
        const int32_t k = ops[4 * o], y = ops[4 * o + 1], z = ops[4 * o + 2], w = ops[4 * o + 3];
        const std::string smp = "sample0 + tm.sample_off";
        const bool st = (k == OP_MAT || k == OP_DIAG) && (w & OPF_PER_SAMPLE) && staged_index.count(z);
        const int si = st ? staged_index[z] : -1;
        s << "    ";
        switch (k) {
            case OP_MAP:
                s << exchange_code(d, cur, y, z, w, rb, false);
                cur = decode_mapping(y, z, w, rb);
                break;
            case OP_MAT:
                if (st)
                    s << "jmat_staged<" << y << ", RB>(pt, xm, staged, " << si << ");\n";
                else
                    s << "jmat<" << y << ", RB>(pt, xm, A, s_mats, " << z << ", " << w << ", " << smp << ");\n";
                break;
            case OP_DIAG:
                if (y & LOC_REG) {
                    if (st)
                        s << "jdiag_staged<" << (y & 7) << ", RB>(pt, xm, staged, " << si << ");\n";
                    else
                        s << "jdiag<" << (y & 7) << ", RB>(pt, xm, A, s_mats, " << z << ", " << w << ", " << smp
                          << ");\n";
                } else {
                    if (st)
                        s << "jdiag_thread_staged<RB>(pt, " << loc_bit(y) << ", staged, " << si << ");\n";
                    else
                        s << "jdiag_thread<RB>(pt, " << loc_bit(y) << ", A, s_mats, " << z << ", " << w << ", "
                          << smp << ");\n";
                }
                break;
            case OP_CX:
                if (z & LOC_REG)
                    s << "jcx<" << y << ", " << (z & 7) << ", RB>(pt, xm);\n";
                else
                    s << "xm ^= (uint32_t)" << loc_bit(z) << " << " << y << ";\n";
                break;
            case OP_CZ: {
                int mask = 0;
                std::string cond;
                for (int32_t loc : {y, z}) {
                    if (loc & LOC_REG) {
                        s << "jmaterialize<" << (loc & 7) << ", RB>(pt, xm); ";
                        mask |= 1 << (loc & 7);
                    } else {
                        cond += (cond.empty() ? "" : " && ") + loc_bit(loc);
                    }
                }
                if (cond.empty())
                    s << "pnegate<" << mask << ", RB>(pt);\n";
                else
                    s << "jnegate_if<" << mask << ", RB>(pt, " << cond << ");\n";
                break;
            }
            case OP_SWAP:
                if (y != z) s << "jswap<" << y << ", " << z << ", RB>(pt, xm);\n";
                else s << "\n";
                break;
            case OP_XMAT:
                s << "jmaterialize<" << y << ", RB>(pt, xm);\n";
                break;
            default:
                s << "// op " << k << " has no forward form\n";
                break;
        }
    }
    s << "  }\n};\n}  // namespace qg\n"
      << "extern \"C\" __global__ void __launch_bounds__(" << fwd_threads(tb, rb) << ", " << fwd_min_blocks(tb, rb)
      << ")\n"
      << "qg_fwd_pass(const __grid_constant__ qg::JobTable<1> jt) {\n"
      << "  qg::fwd_pass_body<" << tb << ", " << rb << ", 1, qg::PassOps>(jt);\n}\n";
    return s.str();
}

// One backward pass as CUDA source: the shared backward body with the pass's
// ops unrolled on psi and lambda, gradient partials at compile-time slots.
std::string bwd_pass_source(const ProgramRun& R, int p) {
    const PassDesc& d = R.bpass[p];
    const int tb = d.tile_bits, rb = kBwdRegBits;
    const int nt = 1 << (tb - rb);
    const int32_t* ops = R.bops + 4 * (size_t)d.op_begin;
    std::ostringstream s;
    s << "#include \"jit_ops.cuh\"\n"
         "namespace qg {\n"
         "struct BwdPassOps {\n"
         "  static constexpr bool kStageOps = false;\n"
         "  template <int TB, int RB>\n"
         "  __device__ __forceinline__ static void apply(PTile<RB>& pt, PTile<RB>& lt, uint32_t& xm, ThreadMap& tm, "
         "const PassDesc& d, const RunArgs& A, const int4*, const int4*, const float4* s_mats, float* pp, float* lp, "
         "int64_t sample0, uint32_t fixed_val, int tid, float* gacc, uint8_t* gsmp) {\n"
         "    constexpr int NT = 1 << (TB - RB);\n"
         "    int swb = tm.sw_base;\n"
         "    (void)swb;\n";
    MapBits cur;
    {
        int32_t y0, z0, w0;
        natural_mapping(tb, rb, y0, z0, w0);
        cur = decode_mapping(y0, z0, w0, rb);
    }
    for (int o = 0; o < d.op_count; ++o) {
        const int32_t k = ops[4 * o], y = ops[4 * o + 1], z = ops[4 * o + 2], w = ops[4 * o + 3];
        const std::string smp = "sample0 + tm.sample_off";
        s << "    ";
        switch (k) {
            case OP_MAP:
                s << exchange_code(d, cur, y, z, w, rb, true);
                cur = decode_mapping(y, z, w, rb);
                break;
            case OP_GRAD:
                s << "jgrad<" << y << ", RB, NT>(pt, lt, xm, " << z << ", gacc, gsmp, " << (w - d.grad_base)
                  << ", tid, tm.sample_off);\n";
                break;
            case OP_MAT:
                if (w & OPF_GRAD)
                    s << "jgrad<" << y << ", RB, NT>(pt, lt, xm, " << ((w >> 8) & 3) << ", gacc, gsmp, "
                      << ((w >> 12) - d.grad_base) << ", tid, tm.sample_off); ";
                s << "jmat2<" << y << ", RB>(pt, lt, xm, A, s_mats, " << z << ", " << w << ", " << smp << ");\n";
                break;
            case OP_DIAG:
                if (y & LOC_REG)
                    s << "jdiag2<" << (y & 7) << ", RB>(pt, lt, xm, A, s_mats, " << z << ", " << w << ", " << smp
                      << ");\n";
                else
                    s << "jdiag_thread2<RB>(pt, lt, " << loc_bit(y) << ", A, s_mats, " << z << ", " << w << ", "
                      << smp << ");\n";
                break;
            case OP_CX:
                if (z & LOC_REG)
                    s << "jcx2<" << y << ", " << (z & 7) << ", RB>(pt, lt, xm);\n";
                else
                    s << "xm ^= (uint32_t)" << loc_bit(z) << " << " << y << ";\n";
                break;
            case OP_CZ: {
                int mask = 0;
                std::string cond;
                for (int32_t loc : {y, z}) {
                    if (loc & LOC_REG) {
                        s << "jmaterialize2<" << (loc & 7) << ", RB>(pt, lt, xm); ";
                        mask |= 1 << (loc & 7);
                    } else {
                        cond += (cond.empty() ? "" : " && ") + loc_bit(loc);
                    }
                }
                if (cond.empty())
                    s << "jnegate2<" << mask << ", RB>(pt, lt);\n";
                else
                    s << "jnegate_if2<" << mask << ", RB>(pt, lt, " << cond << ");\n";
                break;
            }
            case OP_SWAP:
                if (y != z) s << "jswap2<" << y << ", " << z << ", RB>(pt, lt, xm);\n";
                else s << "\n";
                break;
            case OP_XMAT:
                s << "jmaterialize2<" << y << ", RB>(pt, lt, xm);\n";
                break;
            default:
                s << "// op " << k << " has no backward form\n";
                break;
        }
    }
    s << "  }\n};\n}  // namespace qg\n"
      << "extern \"C\" __global__ void __launch_bounds__(" << bwd_threads(tb, rb) << ", 1)\n"
      << "qg_bwd_pass(const qg::PassDesc* __restrict__ passes, const int4* __restrict__ ops_all, int pass_index, "
         "qg::RunArgs A, int store_lam_last, int64_t num_tiles) {\n"
      << "  qg::bwd_pass_body<" << tb << ", " << rb << ", qg::BwdPassOps>(passes, ops_all, pass_index, A, "
         "store_lam_last, num_tiles);\n}\n";
    return s.str();
}

// ------------------------------------------------- compile and cache --

struct Loaded {
    CUmodule mod = nullptr;
    JitKernel k;
};

std::mutex g_cache_mu;
std::map<std::pair<int, std::string>, Loaded> g_cache;  // (device, source) -> module

const char* const kOpts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo", "-DQG_RTC=1"};
constexpr int kNumOpts = (int)(sizeof(kOpts) / sizeof(kOpts[0]));

// Optional on-disk cache of compiled passes: QG_JIT_CACHE_DIR names a
// directory; a pass's cubin is stored under a 64-bit FNV-1a hash of its
// source, the headers it includes, the compile options and the NVRTC
// version.
std::string cache_path(const std::string& src, const char* const* opts, int nopts) {
    const char* dir = getenv("QG_JIT_CACHE_DIR");
    if (!dir || !*dir) return "";
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const std::string& t) {
        for (unsigned char ch : t) {
            h ^= ch;
            h *= 1099511628211ull;
        }
        h ^= 0xff;
        h *= 1099511628211ull;
    };
    mix(src);
    for (int i = 0; i < kJitHeaderCount; ++i) mix(kJitHeaderTexts[i]);  // the kernel body it includes
    for (int i = 0; i < nopts; ++i) mix(opts[i]);
    int major = 0, minor = 0;
    if (nvrtc().version) nvrtc().version(&major, &minor);
    mix(std::to_string(major) + "." + std::to_string(minor));
    char name[64];
    snprintf(name, sizeof(name), "/qg_pass_%016llx_%zu.cubin", (unsigned long long)h, src.size());
    return std::string(dir) + name;
}

bool cache_read(const std::string& path, std::vector<char>& cubin) {
    if (path.empty()) return false;
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return false;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    bool ok = n > 0;
    if (ok) {
        cubin.resize((size_t)n);
        ok = fread(cubin.data(), 1, (size_t)n, f) == (size_t)n;
    }
    fclose(f);
    return ok;
}

void cache_write(const std::string& path, const std::vector<char>& cubin) {
    if (path.empty()) return;
    const std::string tmp = path + ".tmp" + std::to_string((long long)getpid()) + "_" +
                            std::to_string((unsigned long long)std::hash<std::thread::id>()(std::this_thread::get_id()));
    FILE* f = fopen(tmp.c_str(), "wb");
    if (!f) return;
    const bool ok = fwrite(cubin.data(), 1, cubin.size(), f) == cubin.size();
    fclose(f);
    if (ok) rename(tmp.c_str(), path.c_str());
    else remove(tmp.c_str());
}

int compile_source(const std::string& src, std::vector<char>& cubin, std::string& err) {
    const Nvrtc& N = nvrtc();
    const std::string cpath = cache_path(src, kOpts, kNumOpts);
    if (cache_read(cpath, cubin)) return QG_OK;
    nvrtcProgram prog = nullptr;
    nvrtcResult r = N.create(&prog, src.c_str(), "qg_pass.cu", kJitHeaderCount, kJitHeaderTexts, kJitHeaderNames);
    if (r != NVRTC_SUCCESS) {
        err = std::string("nvrtcCreateProgram: ") + N.error_string(r);
        return QG_ECUDA;
    }
    r = N.compile(prog, kNumOpts, kOpts);
    if (r != NVRTC_SUCCESS) {
        size_t n = 0;
        N.log_size(prog, &n);
        std::string log(n, '\0');
        if (n) N.log(prog, &log[0]);
        err = std::string("nvrtcCompileProgram: ") + N.error_string(r) + "\n" + log.substr(0, 4000);
        N.destroy(&prog);
        return QG_ECUDA;
    }
    size_t n = 0;
    N.cubin_size(prog, &n);
    cubin.resize(n);
    N.cubin(prog, cubin.data());
    N.destroy(&prog);
    cache_write(cpath, cubin);
    return QG_OK;
}

int load_cubin(const std::vector<char>& cubin, const char* fname, int smem, int threads, Loaded& out,
               std::string& err) {
    const Driver& D = driver();
    CUresult r = D.load(&out.mod, cubin.data());
    if (r != CUDA_SUCCESS) {
        err = "cuModuleLoadData: " + cu_error(r);
        return QG_ECUDA;
    }
    CUfunction f = nullptr;
    r = D.get_function(&f, out.mod, fname);
    if (r != CUDA_SUCCESS) {
        err = "cuModuleGetFunction: " + cu_error(r);
        return QG_ECUDA;
    }
    r = D.set_attribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, smem);
    if (r != CUDA_SUCCESS) {
        err = "cuFuncSetAttribute: " + cu_error(r);
        return QG_ECUDA;
    }
    int per_sm = 0;
    r = D.occupancy(&per_sm, f, threads, (size_t)smem);
    if (r != CUDA_SUCCESS) {
        err = "cuOccupancyMaxActiveBlocksPerMultiprocessor: " + cu_error(r);
        return QG_ECUDA;
    }
    out.k.fn = (void*)f;
    out.k.per_sm = per_sm < 1 ? 1 : per_sm;
    return QG_OK;
}

// Per-program state: the compiled kernel of every forward pass, per device.
struct ProgramJit {
    std::mutex mu;
    std::map<int, std::vector<JitKernel>> fwd, bwd;  // device -> kernel per pass
};

}  // namespace

static bool jit_kernel(const void* prog, bool backward, int pass, JitKernel* out) {
    ProgramJit* st = (ProgramJit*)program_jit_state(prog);
    if (!st) return false;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    std::lock_guard<std::mutex> lk(st->mu);
    const auto& m = backward ? st->bwd : st->fwd;
    auto it = m.find(dev);
    if (it == m.end() || pass < 0 || pass >= (int)it->second.size()) return false;
    *out = it->second[pass];
    return out->fn != nullptr;
}

bool jit_forward_kernel(const void* prog, int pass, JitKernel* out) { return jit_kernel(prog, false, pass, out); }
bool jit_backward_kernel(const void* prog, int pass, JitKernel* out) { return jit_kernel(prog, true, pass, out); }

int jit_launch(const JitKernel& k, unsigned grid, unsigned block, size_t smem, void* stream, void** params) {
    CUresult r = driver().launch((CUfunction)k.fn, grid, 1, 1, block, 1, 1, (unsigned)smem, (CUstream)stream,
                                 params, nullptr);
    if (r == CUDA_ERROR_INVALID_CONTEXT) {
        // first launch from a thread that has made no runtime call: make the
        // primary context of the current device current and launch again
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaSetDevice(dev) == cudaSuccess)
            r = driver().launch((CUfunction)k.fn, grid, 1, 1, block, 1, 1, (unsigned)smem, (CUstream)stream, params,
                                nullptr);
    }
    if (r != CUDA_SUCCESS) {
        set_error("cuLaunchKernel: " + cu_error(r));
        return QG_ECUDA;
    }
    return QG_OK;
}

void jit_release(void* state) { delete (ProgramJit*)state; }

}  // namespace qg

extern "C" {

int qg_program_compile(qg_program* prog, int flags) {
    using namespace qg;
    if (!prog) return set_error("qg_program_compile: null pointer"), QG_EINVAL;
    const bool load = !(flags & QG_COMPILE_NO_LOAD);
    const bool with_bwd = (flags & QG_COMPILE_BACKWARD) != 0;
    const bool background = (flags & QG_COMPILE_BACKGROUND) != 0;
    const Nvrtc& N = nvrtc();
    if (!N.why.empty()) return set_error("qg_program_compile: " + N.why), QG_ECUDA;
    int dev = -1;
    if (load) {
        const Driver& D = driver();
        if (!D.why.empty()) return set_error("qg_program_compile: " + D.why), QG_ECUDA;
        QG_CUDA_TRY(cudaGetDevice(&dev));
        // a thread that has made no runtime call yet has no current context
        // for the driver calls below: cudaSetDevice makes the device's
        // primary context current on this thread
        QG_CUDA_TRY(cudaSetDevice(dev));
    }
    ProgramRun R;
    program_run_info(prog, &R);
    if (R.reg_bits != 4 && R.reg_bits != 5)
        return set_error("qg_program_compile: reg_bits must be 4 or 5"), QG_EINVAL;

    // one task per pass: forward passes, then (optionally) backward passes
    struct Task {
        bool bwd;
        int pass;
        std::string src;
    };
    std::vector<Task> tasks;
    for (int p = 0; p < R.nfpass; ++p) tasks.push_back({false, p, pass_source(R, p)});
    if (with_bwd)
        for (int p = 0; p < R.nbpass; ++p) tasks.push_back({true, p, bwd_pass_source(R, p)});
    auto name = [](const Task& t) {
        return std::string(t.bwd ? "backward pass " : "pass ") + std::to_string(t.pass);
    };

    // tasks not yet in the process-wide cache compile in parallel
    std::vector<JitKernel> kernels(tasks.size());
    std::vector<size_t> todo;
    {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        for (size_t i = 0; i < tasks.size(); ++i) {
            auto it = g_cache.find({dev, tasks[i].src});
            if (it != g_cache.end())
                kernels[i] = it->second.k;
            else
                todo.push_back(i);
        }
    }
    std::vector<std::vector<char>> cubins(todo.size());
    std::vector<std::string> errs(todo.size());
    std::vector<int> rcs(todo.size(), QG_OK);
    {
        unsigned hw = std::thread::hardware_concurrency();
        if (!hw) hw = 4;
        // a background compile leaves most cores to the caller's other work
        size_t nthreads = std::min<size_t>(todo.size(), background ? std::max(1u, hw / 4) : hw);
        std::vector<std::thread> pool;
        std::mutex qmu;
        size_t next = 0;
        for (size_t t = 0; t < nthreads; ++t)
            pool.emplace_back([&] {
                // background compiles run at a lower scheduling priority (the
                // nice value of a Linux thread is its own)
                if (background) (void)setpriority(PRIO_PROCESS, (id_t)syscall(SYS_gettid), 10);
                for (;;) {
                    size_t i;
                    {
                        std::lock_guard<std::mutex> lk(qmu);
                        if (next >= todo.size()) return;
                        i = next++;
                    }
                    rcs[i] = compile_source(tasks[todo[i]].src, cubins[i], errs[i]);
                }
            });
        for (auto& th : pool) th.join();
    }
    for (size_t i = 0; i < todo.size(); ++i)
        if (rcs[i]) return set_error("qg_program_compile: " + name(tasks[todo[i]]) + ": " + errs[i]), rcs[i];
    if (!load) return QG_OK;
    {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        for (size_t i = 0; i < todo.size(); ++i) {
            const Task& t = tasks[todo[i]];
            auto it = g_cache.find({dev, t.src});
            if (it == g_cache.end()) {
                Loaded L;
                std::string err;
                const int tb = t.bwd ? R.bpass[t.pass].tile_bits : R.fpass[t.pass].tile_bits;
                const int rb = t.bwd ? kBwdRegBits : R.reg_bits;
                const int smem = t.bwd ? bwd_smem_bytes(tb, rb) : fwd_smem_bytes(tb);
                const int threads = t.bwd ? bwd_threads(tb, rb) : fwd_threads(tb, rb);
                int rc = load_cubin(cubins[i], t.bwd ? "qg_bwd_pass" : "qg_fwd_pass", smem, threads, L, err);
                if (rc) return set_error("qg_program_compile: " + name(t) + ": " + err), rc;
                it = g_cache.emplace(std::make_pair(dev, t.src), L).first;
            }
            kernels[todo[i]] = it->second.k;
        }
    }
    ProgramJit* st;
    {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        st = (ProgramJit*)program_jit_state(prog);
        if (!st) {
            st = new ProgramJit();
            program_set_jit_state(prog, st);
        }
    }
    std::lock_guard<std::mutex> lk(st->mu);
    st->fwd[dev] = std::vector<JitKernel>(kernels.begin(), kernels.begin() + R.nfpass);
    if (with_bwd) st->bwd[dev] = std::vector<JitKernel>(kernels.begin() + R.nfpass, kernels.end());
    return QG_OK;
}

int64_t qg_program_pass_source(const qg_program* prog, int backward, int pass, char* host_out, int64_t bytes) {
    using namespace qg;
    if (!prog) return -1;
    ProgramRun R;
    program_run_info(prog, &R);
    if (pass < 0 || pass >= (backward ? R.nbpass : R.nfpass)) return -1;
    const std::string src = backward ? bwd_pass_source(R, pass) : pass_source(R, pass);
    const int64_t need = (int64_t)src.size() + 1;
    if (host_out && bytes >= need) memcpy(host_out, src.c_str(), (size_t)need);
    return need;
}

int qg_program_compiled(const qg_program* prog) {
    qg::JitKernel k;
    if (!prog || !qg::jit_forward_kernel(prog, 0, &k)) return 0;
    return qg::jit_backward_kernel(prog, 0, &k) ? 3 : 1;
}

}  // extern "C"

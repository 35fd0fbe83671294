// Shared helpers for the qandle_gb300 CUDA library (sm_103a).
//
// State layout everywhere: complex64 amplitudes as float2 {re, im}, shaped
// [batch][2^n], row-major and contiguous; qubit q of the reference lives at
// bit (n-1-q) of the basis index (qandle/operators.py:549).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "devmath.cuh"
#include "qandle_gb300.h"

namespace qg {

static_assert(kStatusTimeout == QG_ETIMEOUT, "device copy of the timeout status");

// Last error message of the calling host thread (read through qg_last_error).
void set_error(const std::string& msg);
const char* last_error();

// Status codes are the QG_* macros of qandle_gb300.h:
//   QG_EINVAL   bad argument (shape, qubit index, alignment, size)
//   QG_ECUDA    a CUDA runtime call failed
//   QG_ETIMEOUT a bounded device wait gave up
//   QG_ENOMEM   a caller-provided buffer or budget is too small

#define QG_CHECK_ARG(cond, msg)                                   \
    do {                                                          \
        if (!(cond)) {                                            \
            qg::set_error(std::string(__func__) + ": " + (msg));  \
            return QG_EINVAL;                                 \
        }                                                         \
    } while (0)

#define QG_CUDA_TRY(expr)                                                              \
    do {                                                                               \
        cudaError_t e_ = (expr);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            qg::set_error(std::string(__func__) + ": " #expr ": " + cudaGetErrorString(e_)); \
            return QG_ECUDA;                                                       \
        }                                                                              \
    } while (0)

#define QG_LAUNCH_CHECK() QG_CUDA_TRY(cudaGetLastError())

inline int grid_for(int64_t work, int threads, int64_t cap = 1 << 20) {
    int64_t g = (work + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

}  // namespace qg

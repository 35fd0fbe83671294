// Run-time compiled forward pass kernels (jit.cpp), host interface for the
// launch code in fused.cu.
#pragma once
#include <stddef.h>

namespace qg {

// A compiled forward pass kernel loaded on one device.
struct JitKernel {
    void* fn = nullptr;  // CUfunction
    int per_sm = 0;      // resident CTAs per SM at the pass's shared-memory size
};

// The compiled kernel of forward pass `pass` of `prog` on the current device;
// false when the program has not been compiled for it.
bool jit_forward_kernel(const void* prog, int pass, JitKernel* out);
// The same for backward pass `pass` (compiled with QG_COMPILE_BACKWARD).
bool jit_backward_kernel(const void* prog, int pass, JitKernel* out);

// cuLaunchKernel on `stream`; QG_OK or a status with the error text set.
int jit_launch(const JitKernel& k, unsigned grid, unsigned block, size_t smem, void* stream, void** params);

// Release the per-program state (the compiled modules stay cached).
void jit_release(void* state);

}  // namespace qg

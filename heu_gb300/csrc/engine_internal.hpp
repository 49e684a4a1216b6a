// Internal accessors of the engine for translation units other than
// engine.cu (no C-ABI).
#pragma once
#include <cuda_runtime.h>

#include "../../include/heu_gb300.h"
#include "paillier_kernels.cuh"

namespace hg {

// Looks up a loaded key without allocating.  On success fills the key's
// constants, its limb count S, the context's device and the context's own
// stream and returns HG_OK; otherwise returns an HG_ERR_* code.
int key_view(hg_ctx* ctx, int key_id, KeyConst* kc, int* S, int* device, cudaStream_t* own_stream);

// Records `msg` as the calling thread's last error (read by hg_last_error).
void set_last_error(const char* msg);

// Drops the cached device address of the allocation-free Sum's scratch array
// for `device` (called when a context is created there).
void forget_noalloc_scratch(int device);

}  // namespace hg

// Descriptors of the persistent multi-key batch kernel (batch_kernels.cu),
// shared with the host engine.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "paillier_kernels.cuh"

namespace hg {

enum : int { kBatchEncrypt = 0, kBatchDecrypt = 1, kBatchAdd = 2, kBatchMul = 3 };

struct BatchJob {
  int op;      // kBatch*
  int S;       // 32-bit limbs of n^2 (64 / 128 / 192)
  int wm;      // scalar-mul window
  int pad;
  KeyConst kc;
  SecConst sc;
  const void* in0;  // m (int64) | ct | a | a
  const void* in1;  // r (uint32 limbs) | - | b | k (int64)
  void* out;        // ct | m (int64) | ct | ct
  void* aux;        // - | overflow flags | - | -
  uint64_t count;
};

struct BatchTile {
  uint32_t job;
  uint32_t start;
  uint32_t count;
  uint32_t pad;
};

// (threads per instance) for n^2 with S limbs and (threads per side) for p^2
// with SP limbs, per variant; V = 0 / 1 must match HG_DISPATCH_SV /
// HG_DISPATCH_SPV, V = 2 (latency layout) HG_DISPATCH_SL / HG_DISPATCH_SPL.
__host__ __device__ constexpr int tpi_for(int S, int V) {
  return V == 2 ? 32 : S == 64 ? (V ? 8 : 4) : S == 128 ? (V ? 4 : 8) : (V ? 8 : 16);
}
__host__ __device__ constexpr int tp_for(int SP, int V) {
  return V == 2 ? 16 : SP == 32 ? (V ? 4 : 2) : SP == 64 ? (V ? 8 : 4) : (V ? 4 : 8);
}
// Variant set of the latency layout (short requests).
constexpr int kBatchLatencyVariant = 2;

int batch_resident_blocks(int variant);
// Every variant of the batch kernel prefers the largest shared-memory carveout
// (see server_prefer_shared_carveout).
void batch_prefer_shared_carveout();
int batch_warps_per_block();
cudaError_t launch_batch(int variant, const BatchJob* jobs, const BatchTile* tiles, uint32_t ntiles,
                         uint32_t* counter, uint32_t* scratch, size_t warp_words, uint32_t* err, int grid,
                         cudaStream_t st, size_t dyn_smem = 0);
// Resident blocks per SM of the batch kernel (register-limited).
int batch_blocks_per_sm(int variant);
// Dynamic shared memory that limits the batch kernel to `blocks_per_sm`
// resident blocks per SM (sets the kernel's shared-memory attributes); the
// blocks it keeps free run another launch of the kernel without padding.
size_t batch_smem_cap(int variant, int blocks_per_sm);

}  // namespace hg

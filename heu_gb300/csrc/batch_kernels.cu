// Host-side entry points of the persistent multi-key batch kernel
// (batch_body.cuh): dispatch over the layout variant sets, each compiled in
// its own translation unit (batch_v0.cu, batch_v1.cu, batch_v2.cu).
#include <algorithm>

#include "batch.cuh"

namespace hg {

#define HG_BATCH_DECLARE(V)                                                                                  \
  void batch_carveout_v##V(int pct);                                                                         \
  int batch_resident_blocks_v##V();                                                                          \
  size_t batch_smem_cap_v##V(int blocks_per_sm);                                                             \
  cudaError_t launch_batch_v##V(const BatchJob* jobs, const BatchTile* tiles, uint32_t ntiles,               \
                                uint32_t* counter, uint32_t* scratch, size_t warp_words, uint32_t* err,      \
                                int grid, cudaStream_t st, size_t dyn_smem);
HG_BATCH_DECLARE(0)
HG_BATCH_DECLARE(1)
HG_BATCH_DECLARE(2)

namespace {
constexpr int kWarps = 4;  // warps per block of the batch kernel
}

int batch_resident_blocks(int variant) {
  switch (variant) {
    case 1: return batch_resident_blocks_v1();
    case 2: return batch_resident_blocks_v2();
    default: return batch_resident_blocks_v0();
  }
}

int batch_warps_per_block() { return kWarps; }

void batch_prefer_shared_carveout() {
  batch_carveout_v0(100);
  batch_carveout_v1(100);
  batch_carveout_v2(100);
}

cudaError_t launch_batch(int variant, const BatchJob* jobs, const BatchTile* tiles, uint32_t ntiles,
                         uint32_t* counter, uint32_t* scratch, size_t warp_words, uint32_t* err, int grid,
                         cudaStream_t st, size_t dyn_smem) {
  if (ntiles == 0) return cudaSuccess;
  switch (variant) {
    case 1: return launch_batch_v1(jobs, tiles, ntiles, counter, scratch, warp_words, err, grid, st, dyn_smem);
    case 2: return launch_batch_v2(jobs, tiles, ntiles, counter, scratch, warp_words, err, grid, st, dyn_smem);
    default: return launch_batch_v0(jobs, tiles, ntiles, counter, scratch, warp_words, err, grid, st, dyn_smem);
  }
}

size_t batch_smem_cap(int variant, int blocks_per_sm) {
  if (blocks_per_sm < 1) blocks_per_sm = 1;
  switch (variant) {
    case 1: return batch_smem_cap_v1(blocks_per_sm);
    case 2: return batch_smem_cap_v2(blocks_per_sm);
    default: return batch_smem_cap_v0(blocks_per_sm);
  }
}

int batch_blocks_per_sm(int variant) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return batch_resident_blocks(variant) / (sms > 0 ? sms : 1);
}

}  // namespace hg

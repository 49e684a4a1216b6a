// Persistent multi-key batch kernel: the templates, shared by the
// translation units that instantiate one layout variant set each
// (batch_v0.cu, batch_v1.cu, batch_v2.cu), so the variants compile in
// parallel.
//
// One launch runs a whole batch of jobs of different key sizes (1024, 2048,
// 3072 bits) and operations (encrypt, decrypt, add, scalar mul).  The host
// cuts every job into tiles of a few warp passes and orders them by cost
// (most expensive first); each warp repeatedly takes the next tile from a
// device counter and runs the per-ciphertext body of paillier_ops.cuh for
// the tile's key size.  All key sizes of one launch use the (threads per
// instance, limbs per thread) layouts of variant set V (tpi_for / tp_for):
// V = 0 and 1 are throughput layouts the autotuner picks from, V = 2 the
// latency layout (a whole warp per instance mod n^2, a half warp per side
// mod p^2) that short requests run in.
#pragma once
#include <algorithm>

#include "batch.cuh"
#include "paillier_ops.cuh"

namespace hg {

namespace batch_detail {
constexpr int kBlock = 128;
constexpr int kWarps = kBlock / 32;
constexpr int kYsmWordsPerWarp = 32 * 24;  // 32 * max LP over every variant
}  // namespace batch_detail

template <int V, int S>
__device__ __forceinline__ void run_tile(const BatchJob& job, const BatchTile& tile, uint32_t* ws, uint32_t* ysm,
                                         uint32_t* err) {
  constexpr int TPI = tpi_for(S, V), L = S / TPI;
  const int lane = threadIdx.x & 31;
  const size_t end = (size_t)tile.start + tile.count;
  if (job.op == kBatchDecrypt) {
    constexpr int SP = S / 2;
    constexpr int TP = tp_for(SP, V), LP = SP / TP;
    constexpr int UPW = 32 / (2 * TP);
    const Group<TP> g;
    const int side = (lane / TP) & 1;
    const int unit_w = lane / (2 * TP);
    const int ntab = 1 << (job.sc.wd - 1);
    uint32_t* tb = ws + ((size_t)unit_w * 2 + side) * (size_t)ntab * SP + g.t * LP;
    for (size_t wbase = tile.start; wbase < end; wbase += UPW) {
      const size_t inst = wbase + unit_w;
      const bool active = inst < end;
      decrypt_one<TP, LP>(job.kc, job.sc, (const uint32_t*)job.in0, active ? inst : end - 1, active, side, tb,
                          ysm + unit_w * 2 * SP, (int64_t*)job.out, (uint8_t*)job.aux, nullptr, nullptr, g, err);
    }
    return;
  }
  const Group<TPI> g;
  uint32_t N[L];
  load_slice<L>(N, job.kc.N + g.t * L);
  const int lane_inst = lane / TPI;
  constexpr int IPW = 32 / TPI;
  if (job.op == kBatchEncrypt) {
    for (size_t wbase = tile.start; wbase < end; wbase += IPW) {
      const size_t inst = wbase + lane_inst;
      const bool active = inst < end;
      encrypt_one<TPI, L>(job.kc, EncMode::kEncrypt, (const int64_t*)job.in0, nullptr, nullptr,
                          (const uint32_t*)job.in1, nullptr, (uint32_t*)job.out, active ? inst : end - 1, active, N,
                          g, err);
    }
  } else if (job.op == kBatchAdd) {
    for (size_t wbase = tile.start; wbase < end; wbase += IPW) {
      const size_t inst = wbase + lane_inst;
      const bool active = inst < end;
      add_one<TPI, L>(job.kc, (const uint32_t*)job.in0, (const uint32_t*)job.in1, (uint32_t*)job.out,
                      active ? inst : end - 1, active, N, g, err);
    }
  } else if (job.op == kBatchMul) {
    const int ntab = 1 << (job.wm - 1);
    uint32_t* tb = ws + (size_t)lane_inst * ntab * S + g.t * L;
    for (size_t wbase = tile.start; wbase < end; wbase += IPW) {
      const size_t inst = wbase + lane_inst;
      const bool active = inst < end;
      mul_one<TPI, L>(job.kc, (const uint32_t*)job.in0, (const int64_t*)job.in1, (uint32_t*)job.out,
                      active ? inst : end - 1, active, tb, job.wm, N, g, err);
    }
  }
}

template <int V>
__global__ void __launch_bounds__(batch_detail::kBlock) k_batch(const BatchJob* __restrict__ jobs,
                                                  const BatchTile* __restrict__ tiles, uint32_t ntiles,
                                                  uint32_t* __restrict__ counter, uint32_t* __restrict__ scratch,
                                                  size_t warp_words, uint32_t* err) {
  __shared__ __align__(16) uint32_t ysm[batch_detail::kWarps][batch_detail::kYsmWordsPerWarp];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint32_t* ws = scratch + ((size_t)blockIdx.x * batch_detail::kWarps + wib) * warp_words;
  while (true) {
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(counter, 1u);
    t = __shfl_sync(kFull, t, 0);
    if (t >= ntiles) break;
    const BatchTile tile = tiles[t];
    const BatchJob& job = jobs[tile.job];
    switch (job.S) {
      case 64: run_tile<V, 64>(job, tile, ws, ysm[wib], err); break;
      case 128: run_tile<V, 128>(job, tile, ws, ysm[wib], err); break;
      case 192: run_tile<V, 192>(job, tile, ws, ysm[wib], err); break;
      default: break;
    }
  }
}


template <typename K>
int batch_occupancy_blocks(K kernel) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, batch_detail::kBlock, 0);
  return sms * (per > 0 ? per : 1);
}

// Dynamic shared memory that caps `kernel` at `cap` resident blocks per SM.
template <typename K>
size_t batch_smem_cap_pad(K kernel, int cap) {
  int dev = 0, per_sm = 0, reserved = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  cudaFuncAttributes fa{};
  cudaFuncGetAttributes(&fa, kernel);
  // cap blocks fit in per_sm, cap + 1 do not
  const size_t per_block = (size_t)((double)per_sm / ((double)cap + 0.5));
  const size_t used = fa.sharedSizeBytes + (size_t)reserved;
  const size_t pad = per_block > used ? per_block - used : 0;
  cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pad);
  return pad;
}

void count_launches(uint64_t n);

// The three entry points of one variant set, defined by batch_v<V>.cu.
#define HG_BATCH_VARIANT_ENTRY_POINTS(V)                                                                      \
  void batch_carveout_v##V(int pct) {                                                                       \
    cudaFuncSetAttribute(k_batch<V>, cudaFuncAttributePreferredSharedMemoryCarveout, pct);                  \
  }                                                                                                         \
  int batch_resident_blocks_v##V() { return batch_occupancy_blocks(k_batch<V>); }                          \
  size_t batch_smem_cap_v##V(int blocks_per_sm) { return batch_smem_cap_pad(k_batch<V>, blocks_per_sm); } \
  cudaError_t launch_batch_v##V(const BatchJob* jobs, const BatchTile* tiles, uint32_t ntiles,              \
                                uint32_t* counter, uint32_t* scratch, size_t warp_words, uint32_t* err,     \
                                int grid, cudaStream_t st, size_t dyn_smem) {                               \
    k_batch<V><<<grid, batch_detail::kBlock, dyn_smem, st>>>(jobs, tiles, ntiles, counter, scratch,         \
                                                             warp_words, err);                              \
    count_launches(1);                                                                                      \
    return cudaGetLastError();                                                                              \
  }

}  // namespace hg

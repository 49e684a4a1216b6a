// Allocation-free Sum (hg_dev_sum_noalloc).
//
// Some callers cannot call cudaMalloc: code running under a memory manager
// that owns every device allocation of the process, a serving process whose
// device memory is reserved up front, or a caller that must not add
// allocations while it works.  For them this file keeps the partial products
// of the Sum reduction in a file-scope device array of fixed size instead of
// in buffers the engine allocates on demand.  The array is part of the
// library's device image, so every GPU that loads the library holds it until
// the process exits.
//
// Layout of the array (kScratchBytes = 16 MiB):
//   [0, 256)           error word of the range check (cleared by every call)
//   [256, 256 + H)     partial products, ping
//   [256 + H, 256 + 2H) partial products, pong      (H = half of the rest)
// Every call shares the array and it keeps the last call's contents; calls
// that overlap on the GPU (different streams, or different host threads on
// the same device) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "../../include/heu_gb300.h"
#include "engine_internal.hpp"
#include "paillier_kernels.cuh"

namespace {

constexpr size_t kScratchBytes = 16u << 20;
constexpr size_t kHeadBytes = 256;
constexpr int kMaxDevices = 64;
constexpr int kMaxFirstChunk = 128;

static __device__ __align__(256) uint32_t g_sum_scratch[kScratchBytes / sizeof(uint32_t)];

// Device address of g_sum_scratch per device, resolved by the first call on
// that device (so that first call should come before any stream capture) and
// dropped whenever an engine context is created on the device: a device reset
// unloads the module and invalidates every context, and the new context's
// first allocation-free call resolves the address again.
uint32_t* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

// cudaGetSymbolAddress runs with `device` current (the caller set it).
int scratch_address(int device, uint32_t** out) {
  if (device < 0 || device >= kMaxDevices) return HG_ERR_INVALID;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (g_scratch_addr[device] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_sum_scratch);
    if (e != cudaSuccess || p == nullptr) return HG_ERR_CUDA;
    g_scratch_addr[device] = static_cast<uint32_t*>(p);
  }
  *out = g_scratch_addr[device];
  return HG_OK;
}

size_t half_capacity(int S) { return (kScratchBytes - kHeadBytes) / (size_t)(4 * S) / 2; }

// Puts the caller's current device back on every return path.
struct RestoreDevice {
  int device = -1;
  RestoreDevice() {
    if (cudaGetDevice(&device) != cudaSuccess) device = -1;
  }
  ~RestoreDevice() {
    int now = -1;
    if (device >= 0 && cudaGetDevice(&now) == cudaSuccess && now != device) cudaSetDevice(device);
  }
};

}  // namespace

namespace hg {

void forget_noalloc_scratch(int device) {
  if (device < 0 || device >= kMaxDevices) return;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  g_scratch_addr[device] = nullptr;
}

}  // namespace hg

extern "C" int hg_dev_sum_noalloc(hg_ctx* ctx, int key_id, const uint32_t* a, size_t count, uint32_t* out,
                                  void* stream) {
  if (!ctx || !a || !out) {
    hg::set_last_error("hg_dev_sum_noalloc: null argument");
    return HG_ERR_INVALID;
  }
  hg::KeyConst kc;
  int S = 0, device = 0;
  cudaStream_t own = nullptr;
  int rc = hg::key_view(ctx, key_id, &kc, &S, &device, &own);
  if (rc != HG_OK) {
    hg::set_last_error("hg_dev_sum_noalloc: unknown key id");
    return rc;
  }
  if (count == 0) {
    hg::set_last_error("you cannot sum an empty tensor");
    return HG_ERR_INVALID;
  }
  const size_t half = half_capacity(S);
  if (count > (size_t)kMaxFirstChunk * half) {
    hg::set_last_error(
        "hg_dev_sum_noalloc: count exceeds the fixed scratch (at most 128 * floor((16 MiB - 256) / (8 * S)) "
        "ciphertexts: 4,194,176 / 2,097,024 / 1,398,016 for 1024 / 2048 / 3072-bit keys); use hg_dev_sum");
    return HG_ERR_INVALID;
  }
  const RestoreDevice keep;
  if (cudaSetDevice(device) != cudaSuccess) {
    hg::set_last_error("hg_dev_sum_noalloc: cudaSetDevice failed");
    return HG_ERR_CUDA;
  }
  uint32_t* base = nullptr;
  rc = scratch_address(device, &base);
  if (rc != HG_OK) {
    hg::set_last_error("hg_dev_sum_noalloc: cudaGetSymbolAddress failed");
    return rc;
  }
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : own;
  uint32_t* err = base;
  uint32_t* buf[2] = {base + kHeadBytes / 4, base + kHeadBytes / 4 + half * (size_t)S};
  if (cudaMemsetAsync(err, 0, sizeof(uint32_t), st) != cudaSuccess) {
    hg::set_last_error("hg_dev_sum_noalloc: clearing the error word failed");
    return HG_ERR_CUDA;
  }
  cudaError_t ce = cudaSuccess;
  if (count == 1) {
    ce = cudaMemcpyAsync(out, a, (size_t)S * 4, cudaMemcpyDeviceToDevice, st);
  } else {
    const uint32_t* cur = a;
    size_t n = count;
    int which = 0;
    bool first = true;
    const size_t target = (size_t)std::max(1, hg_device_sm_count(ctx) * 4 * hg::instances_per_block(S, kc.variant));
    while (n > 1 && ce == cudaSuccess) {
      size_t chunk;
      if (first) {
        chunk = std::max<size_t>(2, (n + half - 1) / half);  // output fits one half
      } else {
        chunk = std::min<size_t>(64, std::max<size_t>(2, (n + target - 1) / target));
      }
      first = false;
      const size_t outn = (n + chunk - 1) / chunk;
      uint32_t* dst = (outn == 1) ? out : buf[which];
      ce = hg::launch_reduce(S, kc, cur, n, (int)chunk, dst, err, st);
      cur = dst;
      n = outn;
      which ^= 1;
    }
  }
  if (ce != cudaSuccess) {
    hg::set_last_error("hg_dev_sum_noalloc: kernel launch failed");
    return HG_ERR_CUDA;
  }
  uint32_t bits = 0;
  if (cudaMemcpyAsync(&bits, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    hg::set_last_error("hg_dev_sum_noalloc: CUDA error");
    return HG_ERR_CUDA;
  }
  if (bits & hg::kErrCtRange) {
    hg::set_last_error("Invalid ciphertext: value >= n^2");
    return HG_ERR_CT_RANGE;
  }
  return HG_OK;
}

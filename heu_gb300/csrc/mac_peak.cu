// Integer multiply-accumulate throughput probe (the roofline denominator for
// the Montgomery kernels).  Pure register work, no memory traffic:
//   pattern 0: 32x32->64 MACs as carry chains of mad.lo.cc / madc.hi.cc
//              (2 instructions per MAC);
//   pattern 1: 32x32->64 MACs as mad.wide.u32 into 64-bit accumulators.
// Reported as MACs per second over the whole device.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/heu_gb300_probe.h"
#include "mont.cuh"

namespace {

constexpr int kRowL = 16;

// One row of carry-chained 32x32->64 MACs: T (+ carry words) += x * y.
__device__ __forceinline__ void row_chain(uint32_t (&T)[kRowL], uint32_t& c0, uint32_t& c1,
                                          const uint32_t (&x)[kRowL], uint32_t y) {
  T[0] = hg::mad_lo_cc(x[0], y, T[0]);
#pragma unroll
  for (int j = 1; j < kRowL; ++j) T[j] = hg::madc_lo_cc(x[j], y, T[j]);
  c0 = hg::addc_cc(c0, 0u);
  c1 = hg::addc(c1, 0u);
  T[1] = hg::mad_hi_cc(x[0], y, T[1]);
#pragma unroll
  for (int j = 1; j < kRowL - 1; ++j) T[j + 1] = hg::madc_hi_cc(x[j], y, T[j + 1]);
  c0 = hg::madc_hi_cc(x[kRowL - 1], y, c0);
  c1 = hg::addc(c1, 0u);
}

__global__ void __launch_bounds__(256) k_mac_chain(uint32_t* sink, uint32_t seed, int iters) {
  uint32_t x[kRowL], T[kRowL];
#pragma unroll
  for (int j = 0; j < kRowL; ++j) {
    x[j] = seed * (threadIdx.x + 3u * j + 1u) + j;
    T[j] = 0;
  }
  uint32_t c0 = 0, c1 = 0, y = seed ^ threadIdx.x;
#pragma unroll 1
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      row_chain(T, c0, c1, x, y);
      y ^= T[r];
    }
  }
  uint32_t acc = c0 ^ c1;
#pragma unroll
  for (int j = 0; j < kRowL; ++j) acc ^= T[j];
  if (acc == 0x9e3779b9u) sink[threadIdx.x] = acc;  // keep the work alive
}

__global__ void __launch_bounds__(256) k_mac_wide(uint32_t* sink, uint32_t seed, int iters) {
  uint32_t x[kRowL];
  uint64_t acc[kRowL];
#pragma unroll
  for (int j = 0; j < kRowL; ++j) {
    x[j] = seed * (threadIdx.x + 3u * j + 1u) + j;
    acc[j] = 0;
  }
  uint32_t y = seed ^ threadIdx.x;
#pragma unroll 1
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
#pragma unroll
      for (int j = 0; j < kRowL; ++j) {
        asm volatile("mad.wide.u32 %0, %1, %2, %3;" : "=l"(acc[j]) : "r"(x[j]), "r"(y), "l"(acc[j]));
      }
      y ^= (uint32_t)acc[r];
    }
  }
  uint64_t a = 0;
#pragma unroll
  for (int j = 0; j < kRowL; ++j) a ^= acc[j];
  if (a == 0x9e3779b97f4a7c15ull) sink[threadIdx.x] = (uint32_t)a;
}

}  // namespace

extern "C" int hg_probe_mac_peak(int device, int pattern, double* macs_per_second, double* seconds) {
  if (!macs_per_second) return 1;
  if (cudaSetDevice(device) != cudaSuccess) return 5;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  uint32_t* sink = nullptr;
  if (cudaMalloc(&sink, 256 * sizeof(uint32_t)) != cudaSuccess) return 4;
  const int threads = 256, blocks = sms * 8, iters = 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto launch = [&]() {
    if (pattern == 0)
      k_mac_chain<<<blocks, threads>>>(sink, 0x12345u, iters);
    else
      k_mac_wide<<<blocks, threads>>>(sink, 0x12345u, iters);
  };
  launch();  // warm-up
  cudaEventRecord(e0);
  const int reps = 40;  // about half a second of sustained load
  for (int i = 0; i < reps; ++i) launch();
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess) return 5;
  const double macs = (double)reps * blocks * threads * (double)iters * 4.0 * kRowL;
  *macs_per_second = macs / (ms * 1e-3);
  if (seconds) *seconds = ms * 1e-3 / reps;
  return 0;
}

extern "C" int hg_probe_host_copy(int device, void* host, size_t bytes, int dir, int* mem_type, double* gbs) {
  if (!host || !mem_type || !gbs || bytes == 0) return 1;
  if (cudaSetDevice(device) != cudaSuccess) return 2;
  cudaPointerAttributes pa{};
  *mem_type = (cudaPointerGetAttributes(&pa, host) == cudaSuccess) ? (int)pa.type : -1;
  cudaGetLastError();
  void* d = nullptr;
  if (cudaMalloc(&d, bytes) != cudaSuccess) return 3;
  cudaStream_t st;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  // one untimed copy, then the timed one
  for (int it = 0; it < 2; ++it) {
    if (it) cudaEventRecord(a, st);
    if (dir == 0)
      cudaMemcpyAsync(d, host, bytes, cudaMemcpyHostToDevice, st);
    else
      cudaMemcpyAsync(host, d, bytes, cudaMemcpyDeviceToHost, st);
    if (it) cudaEventRecord(b, st);
  }
  const cudaError_t e = cudaEventSynchronize(b);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a, b);
  *gbs = ms > 0.0f ? (double)bytes / (ms * 1e-3) / 1e9 : 0.0;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaStreamDestroy(st);
  cudaFree(d);
  return e == cudaSuccess ? 0 : 4;
}


// heu.numpy reductions beyond Sum: FeatureWiseBucketSum building blocks.
//
// FeatureWiseBucketSum (numpy/evaluator.cc:378-458) multiplies, for every
// feature f and bucket b, the ciphertexts of the rows whose bin id is b.  On
// the device this is a counting sort of row indices by (feature, bin)
// followed by a segmented product: every segment (one bucket of one feature)
// is cut into chunks of at most C elements, one group of lanes multiplies a
// chunk, and the chunk products are reduced again level by level until each
// segment holds one ciphertext.  Modular multiplication is commutative and
// associative, so the result does not depend on the order the sort produces.
#include <algorithm>

#include "mont.cuh"
#include "paillier_kernels.cuh"

namespace hg {

namespace {
constexpr int kBlock = 128;
}

// ---------------------------------------------------------------------------
// counting sort of rows by (feature, bin)
// ---------------------------------------------------------------------------
__global__ void k_bin_hist(const uint8_t* __restrict__ om, size_t rows, int F, int B, uint32_t* __restrict__ cnt,
                           uint32_t* err) {
  extern __shared__ uint32_t h[];
  const int f = blockIdx.y;
  for (int b = threadIdx.x; b < B; b += blockDim.x) h[b] = 0;
  __syncthreads();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (size_t)gridDim.x * blockDim.x) {
    const int bin = om[i * F + f];
    if (bin >= B) {
      atomicOr(err, kErrBinRange);
    } else {
      atomicAdd(&h[bin], 1u);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < B; b += blockDim.x)
    if (h[b]) atomicAdd(&cnt[(size_t)f * B + b], h[b]);
}

__global__ void k_bin_scatter(const uint8_t* __restrict__ om, size_t rows, int F, int B,
                              uint32_t* __restrict__ cursor, uint32_t* __restrict__ idx) {
  const int f = blockIdx.y;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (size_t)gridDim.x * blockDim.x) {
    const int bin = om[i * F + f];
    if (bin < B) {
      const uint32_t pos = atomicAdd(&cursor[(size_t)f * B + bin], 1u);
      idx[pos] = (uint32_t)i;
    }
  }
}

// out[0] = 0, out[i+1] = in[0] + ... + in[i]; one block, sequential tiles.
__global__ void k_scan_exclusive(const uint32_t* __restrict__ in, size_t n, uint32_t* __restrict__ out) {
  __shared__ uint32_t tile[1024];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) {
    carry = 0;
    out[0] = 0;
  }
  __syncthreads();
  for (size_t base = 0; base < n; base += 1024) {
    const size_t i = base + threadIdx.x;
    tile[threadIdx.x] = i < n ? in[i] : 0u;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      const uint32_t v = threadIdx.x >= (unsigned)off ? tile[threadIdx.x - off] : 0u;
      __syncthreads();
      tile[threadIdx.x] += v;
      __syncthreads();
    }
    if (i < n) out[i + 1] = carry + tile[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 1023) carry += tile[1023];
    __syncthreads();
  }
}

// chunks per segment: ceil(len / C)
__global__ void k_seg_chunks(const uint32_t* __restrict__ offs, int nseg, int C, uint32_t* __restrict__ nch) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nseg) {
    const uint32_t len = offs[s + 1] - offs[s];
    nch[s] = (len + C - 1) / C;
  }
}

// ---------------------------------------------------------------------------
// one level of the segmented product
// element p of the level input is vals[((idx ? idx[p] : p) * stride + voff) * S]
// ---------------------------------------------------------------------------
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_seg_reduce(KeyConst kc, const uint32_t* __restrict__ vals,
                                                       size_t stride, size_t voff, const uint32_t* __restrict__ idx,
                                                       const uint32_t* __restrict__ offs_in,
                                                       const uint32_t* __restrict__ offs_out, int nseg, int C,
                                                       uint32_t* __restrict__ out, size_t upper, uint32_t* err) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t k = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  if (wfirst >= upper) return;
  const uint32_t total = offs_out[nseg];
  const bool active = k < total;
  // segment of chunk k: last s with offs_out[s] <= k (segments without chunks are skipped)
  int lo = 0, hi = nseg - 1;
  const uint32_t kk = active ? (uint32_t)k : 0u;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (offs_out[mid] <= kk) lo = mid; else hi = mid - 1;
  }
  const int s = lo;
  const uint32_t j = kk - offs_out[s];
  const uint32_t start = offs_in[s] + j * (uint32_t)C;
  const uint32_t end = min(start + (uint32_t)C, offs_in[s + 1]);
  uint32_t N[L], acc[L];
  load_slice<L>(N, kc.N + g.t * L);
  auto elem = [&](uint32_t p) -> const uint32_t* {
    const size_t e = idx ? (size_t)idx[p] : (size_t)p;
    return vals + (e * stride + voff) * S;
  };
  const bool has = active && start < end;
  load_slice<L>(acc, (has ? elem(start) : kc.R1) + g.t * L);
  if (idx) {
    // level 1 reads the caller's ciphertexts: validate them (< n^2)
    uint32_t d[L];
    const bool bad = sub_full<TPI, L>(d, acc, N, g) == 0u;
    if (has && bad && g.t == 0) atomicOr(err, kErrCtRange);
  }
#pragma unroll 1
  for (int q = 1; q < C; ++q) {
    const uint32_t p = start + (uint32_t)q;
    const bool valid = has && p < end;
    if (!__any_sync(kFull, valid)) break;
    uint32_t B[L];
    load_slice<L>(B, (valid ? elem(p) : kc.R1) + g.t * L);
    if (idx) {
      uint32_t d[L];
      const bool bad = sub_full<TPI, L>(d, B, N, g) == 0u;
      if (valid && bad && g.t == 0) atomicOr(err, kErrCtRange);
    }
    mont_mul<TPI, L>(acc, acc, B, N, kc.np, g);
  }
  if (active) store_slice<L>(out + k * S + g.t * L, acc);
}

// out[s * ostride + ooff] = segment s's single element, or the Montgomery
// identity (GetZero, numpy/evaluator.h:84-87) for an empty segment.
template <int S>
__global__ void k_seg_finalize(const uint32_t* __restrict__ vals, const uint32_t* __restrict__ offs, int nseg,
                               const uint32_t* __restrict__ R1, uint32_t* __restrict__ out, size_t ostride,
                               size_t ooff) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t s = t / S, w = t % S;
  if (s >= (size_t)nseg) return;
  const bool empty = offs[s + 1] == offs[s];
  out[(s * ostride + ooff) * S + w] = empty ? R1[w] : vals[(size_t)offs[s] * S + w];
}

// cumsum over the buckets of each feature (numpy/evaluator.cc:444-449):
// bucket b becomes the product of buckets 0..b, one group per feature.
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_bucket_cumsum(KeyConst kc, uint32_t* __restrict__ out, int F, int B,
                                                          size_t ostride, size_t ooff) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t f = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  if (wfirst >= (size_t)F) return;
  const bool active = f < (size_t)F;
  const size_t ff = active ? f : F - 1;
  uint32_t N[L], acc[L], x[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(acc, out + ((ff * B) * ostride + ooff) * S + g.t * L);
#pragma unroll 1
  for (int b = 1; b < B; ++b) {
    uint32_t* p = out + ((ff * B + b) * ostride + ooff) * S + g.t * L;
    load_slice<L>(x, p);
    mont_mul<TPI, L>(acc, acc, x, N, kc.np, g);
    if (active) store_slice<L>(p, acc);
  }
}

// ---------------------------------------------------------------------------
#define HG_DISPATCH_S2(S, ...)                                          \
  switch (S) {                                                          \
    case 64: { constexpr int TPI = 4, L = 16; __VA_ARGS__; } break;     \
    case 128: { constexpr int TPI = 8, L = 16; __VA_ARGS__; } break;    \
    case 192: { constexpr int TPI = 16, L = 12; __VA_ARGS__; } break;   \
    default: return cudaErrorInvalidValue;                              \
  }

cudaError_t launch_bin_sort(const uint8_t* om, size_t rows, int F, int B, uint32_t* cnt, uint32_t* offs,
                            uint32_t* cursor, uint32_t* idx, uint32_t* err, cudaStream_t st) {
  const size_t nseg = (size_t)F * B;
  cudaError_t e = cudaMemsetAsync(cnt, 0, nseg * 4, st);
  if (e != cudaSuccess) return e;
  const unsigned gx = (unsigned)std::min<size_t>((rows + 255) / 256, 256);
  k_bin_hist<<<dim3(gx, F), 256, B * sizeof(uint32_t), st>>>(om, rows, F, B, cnt, err);
  k_scan_exclusive<<<1, 1024, 0, st>>>(cnt, nseg, offs);
  e = cudaMemcpyAsync(cursor, offs, nseg * 4, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return e;
  k_bin_scatter<<<dim3(gx, F), 256, 0, st>>>(om, rows, F, B, cursor, idx);
  return cudaGetLastError();
}

cudaError_t launch_seg_level(int S, const KeyConst& kc, const uint32_t* vals, size_t stride, size_t voff,
                             const uint32_t* idx, const uint32_t* offs_in, int nseg, int C, uint32_t* nch,
                             uint32_t* offs_out, uint32_t* out, size_t upper, uint32_t* err, cudaStream_t st) {
  k_seg_chunks<<<(nseg + 255) / 256, 256, 0, st>>>(offs_in, nseg, C, nch);
  k_scan_exclusive<<<1, 1024, 0, st>>>(nch, (size_t)nseg, offs_out);
  HG_DISPATCH_S2(S, {
    const size_t ipb = kBlock / TPI;
    const unsigned blocks = (unsigned)((upper + ipb - 1) / ipb);
    k_seg_reduce<TPI, L><<<blocks, kBlock, 0, st>>>(kc, vals, stride, voff, idx, offs_in, offs_out, nseg, C, out,
                                                   upper, err);
  });
  return cudaGetLastError();
}

cudaError_t launch_seg_finalize(int S, const uint32_t* vals, const uint32_t* offs, int nseg, const uint32_t* R1,
                                uint32_t* out, size_t ostride, size_t ooff, cudaStream_t st) {
  const size_t total = (size_t)nseg * S;
  const unsigned blocks = (unsigned)((total + 255) / 256);
  switch (S) {
    case 64: k_seg_finalize<64><<<blocks, 256, 0, st>>>(vals, offs, nseg, R1, out, ostride, ooff); break;
    case 128: k_seg_finalize<128><<<blocks, 256, 0, st>>>(vals, offs, nseg, R1, out, ostride, ooff); break;
    case 192: k_seg_finalize<192><<<blocks, 256, 0, st>>>(vals, offs, nseg, R1, out, ostride, ooff); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_bucket_cumsum(int S, const KeyConst& kc, uint32_t* out, int F, int B, size_t ostride,
                                 size_t ooff, cudaStream_t st) {
  HG_DISPATCH_S2(S, {
    const size_t ipb = kBlock / TPI;
    k_bucket_cumsum<TPI, L><<<(unsigned)((F + ipb - 1) / ipb), kBlock, 0, st>>>(kc, out, F, B, ostride, ooff);
  });
  return cudaGetLastError();
}

}  // namespace hg

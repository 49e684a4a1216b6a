// HEU's wire format for ciphertext matrices, packed and unpacked on the GPU.
//
// DenseMatrix<Ciphertext>::Serialize (heu/library/numpy/matrix.h:221-262)
// writes a msgpack array [rows, cols, ndim, [e_0 .. e_{n-1}]] whose items are
// msgpack str objects; item i holds the ciphertext's HeObject::Serialize
// bytes (util/he_object.h:27-36: msgpack of the class, which is
// MSGPACK_DEFINE(c_) = a one-element array, paillier_zahlen/ciphertext.h:38,
// ou/ciphertext.h:38) followed by the schema value as a little-endian size_t
// (phe/base/serializable_types.cc:49-69).  The BigInt field c_ is written as
// a msgpack bin of its little-endian magnitude without leading zero bytes.
//
// Packing is byte work bound by HBM: one warp per ciphertext finds its
// length, a three-kernel exclusive scan places the items, and one warp per
// ciphertext writes its item with consecutive lanes on consecutive bytes.
// Unpacking takes the item offsets (found by a host walk over the headers)
// and turns each item back into S limbs.
#include <cstdint>

#include "paillier_kernels.cuh"

namespace hg {

void count_launches(uint64_t n);

namespace {

constexpr int kWarpsPerBlock = 8;
constexpr int kScanBlock = 1024;

// Item k of the column-major DenseMatrix order (matrix.h:159-162) is element
// (k % rows, k / rows); in a row-major array that is (k % rows) * cols + k / rows.
__device__ __forceinline__ size_t elem_of_item(size_t k, size_t rows, size_t cols, int row_major) {
  return row_major ? (k % rows) * cols + k / rows : k;
}

__device__ __forceinline__ int bin_header_len(uint32_t b) { return b < 256u ? 2 : (b < 65536u ? 3 : 5); }
__device__ __forceinline__ int str_header_len(uint64_t l) {
  return l < 32u ? 1 : (l < 256u ? 2 : (l < 65536u ? 3 : 5));
}

// Per ciphertext: magnitude bytes and the item's total bytes (str header
// included).
__global__ void k_wire_sizes(const uint32_t* __restrict__ ct, size_t count, size_t rows, size_t cols, int row_major,
                             int S, uint32_t* __restrict__ mag_bytes, uint64_t* __restrict__ item_bytes) {
  const int lane = threadIdx.x & 31;
  const size_t i = (size_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (i >= count) return;
  const uint32_t* c = ct + elem_of_item(i, rows, cols, row_major) * (size_t)S;
  int top = -1;
  for (int j = lane; j < S; j += 32)
    if (c[j] != 0u) top = j;
  top = __reduce_max_sync(0xffffffffu, top + 1) - 1;
  if (lane == 0) {
    uint32_t b = 0;
    if (top >= 0) b = (uint32_t)top * 4u + (uint32_t)((32 - __clz(c[top]) + 7) / 8);
    const uint64_t inner = 1u + (uint64_t)bin_header_len(b) + b + 8u;  // fixarray(1), bin, schema
    mag_bytes[i] = b;
    item_bytes[i] = (uint64_t)str_header_len(inner) + inner;
  }
}

// Exclusive scan of v within blocks of kScanBlock; block totals to bsum.
__global__ void __launch_bounds__(kScanBlock) k_scan_local(uint64_t* __restrict__ v, size_t count,
                                                           uint64_t* __restrict__ bsum) {
  __shared__ uint64_t warp_sum[kScanBlock / 32];
  const size_t i = (size_t)blockIdx.x * kScanBlock + threadIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t x = i < count ? v[i] : 0u;
  uint64_t s = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint64_t y = __shfl_up_sync(0xffffffffu, s, d);
    if (lane >= d) s += y;
  }
  if (lane == 31) warp_sum[wid] = s;
  __syncthreads();
  if (wid == 0) {
    uint64_t w = warp_sum[lane];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint64_t y = __shfl_up_sync(0xffffffffu, w, d);
      if (lane >= d) w += y;
    }
    warp_sum[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  const uint64_t before = (wid > 0 ? warp_sum[wid - 1] : 0u) + s - x;
  if (i < count) v[i] = before;
  if (threadIdx.x == kScanBlock - 1) bsum[blockIdx.x] = warp_sum[31];
}

// Exclusive scan of the block totals (one block, tiles of kScanBlock with a
// running carry); the grand total goes to bsum[nb].
__global__ void __launch_bounds__(kScanBlock) k_scan_totals(uint64_t* __restrict__ bsum, size_t nb) {
  __shared__ uint64_t warp_sum[kScanBlock / 32];
  __shared__ uint64_t carry;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0u;
  __syncthreads();
  for (size_t base = 0; base < nb; base += kScanBlock) {
    const size_t i = base + threadIdx.x;
    const uint64_t x = i < nb ? bsum[i] : 0u;
    uint64_t s = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint64_t y = __shfl_up_sync(0xffffffffu, s, d);
      if (lane >= d) s += y;
    }
    if (lane == 31) warp_sum[wid] = s;
    __syncthreads();
    if (wid == 0) {
      uint64_t w = warp_sum[lane];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, w, d);
        if (lane >= d) w += y;
      }
      warp_sum[lane] = w;
    }
    __syncthreads();
    const uint64_t c = carry;
    if (i < nb) bsum[i] = c + (wid > 0 ? warp_sum[wid - 1] : 0u) + s - x;
    __syncthreads();
    if (threadIdx.x == 0) carry = c + warp_sum[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) bsum[nb] = carry;
}

__device__ __forceinline__ void put_be(uint8_t* p, uint64_t v, int n) {
  for (int k = 0; k < n; ++k) p[k] = (uint8_t)(v >> (8 * (n - 1 - k)));
}

// One warp per ciphertext writes its item at base + its offset.
__global__ void k_wire_write(const uint32_t* __restrict__ ct, size_t count, size_t rows, size_t cols, int row_major,
                             int S, const uint32_t* __restrict__ mag_bytes, const uint64_t* __restrict__ offs,
                             const uint64_t* __restrict__ bsum, uint64_t schema, uint8_t* __restrict__ out,
                             size_t base) {
  const int lane = threadIdx.x & 31;
  const size_t i = (size_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (i >= count) return;
  const uint32_t b = mag_bytes[i];
  const uint64_t inner = 1u + (uint64_t)bin_header_len(b) + b + 8u;
  const int sh = str_header_len(inner), bh = bin_header_len(b);
  uint8_t* p = out + base + offs[i] + bsum[i / kScanBlock];
  if (lane == 0) {
    if (sh == 1) {
      p[0] = (uint8_t)(0xa0u | (uint32_t)inner);
    } else {
      p[0] = sh == 2 ? 0xd9 : (sh == 3 ? 0xda : 0xdb);
      put_be(p + 1, inner, sh - 1);
    }
    uint8_t* q = p + sh;
    q[0] = 0x91;  // fixarray(1): MSGPACK_DEFINE(c_)
    q[1] = bh == 2 ? 0xc4 : (bh == 3 ? 0xc5 : 0xc6);
    put_be(q + 2, b, bh - 1);
  }
  const uint32_t* c = ct + elem_of_item(i, rows, cols, row_major) * (size_t)S;
  uint8_t* m = p + sh + 1 + bh;
  for (uint32_t j = lane; j < b; j += 32) m[j] = (uint8_t)(c[j >> 2] >> (8 * (j & 3)));
  if (lane < 8) m[b + lane] = (uint8_t)(schema >> (8 * lane));
}

// One warp per item: bytes [offs[i], offs[i] + lens[i]) of buf -> S limbs.
__global__ void k_wire_read(const uint8_t* __restrict__ buf, const uint64_t* __restrict__ offs,
                            const uint64_t* __restrict__ lens, size_t count, size_t rows, size_t cols, int row_major,
                            int S, uint64_t schema, uint32_t* __restrict__ out, uint32_t* err) {
  const int lane = threadIdx.x & 31;
  const size_t i = (size_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (i >= count) return;
  const uint8_t* p = buf + offs[i];
  const uint64_t len = lens[i];
  uint32_t* o = out + elem_of_item(i, rows, cols, row_major) * (size_t)S;
  // header checks (every lane reads the same bytes)
  bool ok = len >= 1u + 2u + 8u && p[0] == 0x91;
  uint64_t b = 0;
  int bh = 0;
  if (ok) {
    const uint8_t t = p[1];
    bh = t == 0xc4 ? 2 : (t == 0xc5 ? 3 : (t == 0xc6 ? 5 : 0));
    ok = bh != 0 && len >= 1u + (uint64_t)bh + 8u;
    if (ok) {
      for (int k = 1; k < bh; ++k) b = (b << 8) | p[1 + k];
      ok = 1u + (uint64_t)bh + b + 8u == len && b <= 4u * (uint64_t)S;
    }
  }
  if (ok) ok = p[len - 8] == (uint8_t)schema;  // serializable_types.cc:117 reads the low byte
  if (!ok) {
    if (lane == 0) atomicOr(err, kErrFormat);
    for (int j = lane; j < S; j += 32) o[j] = 0u;
    return;
  }
  const uint8_t* m = p + 1 + bh;
  for (int j = lane; j < S; j += 32) {
    uint32_t v = 0u;
    for (int k = 3; k >= 0; --k) {
      const uint64_t at = 4u * (uint64_t)j + (uint64_t)k;
      v = (v << 8) | (at < b ? m[at] : 0u);
    }
    o[j] = v;
  }
}

}  // namespace

size_t wire_scratch_words(size_t count) {
  const size_t nb = (count + kScanBlock - 1) / kScanBlock;
  return count /* item bytes */ + nb + 1 /* block totals + grand total */;
}

cudaError_t launch_wire_size(const uint32_t* ct, size_t rows, size_t cols, int row_major, int S, uint32_t* mag_bytes,
                             uint64_t* scratch, uint64_t* total_dev, cudaStream_t st) {
  const size_t count = rows * cols;
  if (count == 0) return cudaMemsetAsync(total_dev, 0, sizeof(uint64_t), st);
  const size_t nb = (count + kScanBlock - 1) / kScanBlock;
  uint64_t* items = scratch;
  uint64_t* bsum = scratch + count;
  const unsigned g = (unsigned)((count + kWarpsPerBlock - 1) / kWarpsPerBlock);
  k_wire_sizes<<<g, 32 * kWarpsPerBlock, 0, st>>>(ct, count, rows, cols, row_major, S, mag_bytes, items);
  k_scan_local<<<(unsigned)nb, kScanBlock, 0, st>>>(items, count, bsum);
  k_scan_totals<<<1, kScanBlock, 0, st>>>(bsum, nb);
  count_launches(3);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(total_dev, bsum + nb, sizeof(uint64_t), cudaMemcpyDeviceToDevice, st);
}

cudaError_t launch_wire_write(const uint32_t* ct, size_t rows, size_t cols, int row_major, int S, uint64_t schema,
                              const uint32_t* mag_bytes, const uint64_t* scratch, uint8_t* out, size_t base,
                              cudaStream_t st) {
  const size_t count = rows * cols;
  if (count == 0) return cudaSuccess;
  const unsigned g = (unsigned)((count + kWarpsPerBlock - 1) / kWarpsPerBlock);
  k_wire_write<<<g, 32 * kWarpsPerBlock, 0, st>>>(ct, count, rows, cols, row_major, S, mag_bytes, scratch,
                                                   scratch + count, schema, out, base);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_wire_unpack(const uint8_t* buf, const uint64_t* offs, const uint64_t* lens, size_t rows,
                               size_t cols, int row_major, int S, uint64_t schema, uint32_t* out, uint32_t* err,
                               cudaStream_t st) {
  const size_t count = rows * cols;
  if (count == 0) return cudaSuccess;
  const unsigned g = (unsigned)((count + kWarpsPerBlock - 1) / kWarpsPerBlock);
  k_wire_read<<<g, 32 * kWarpsPerBlock, 0, st>>>(buf, offs, lens, count, rows, cols, row_major, S, schema, out, err);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace hg

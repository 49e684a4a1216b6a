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
// Packing is byte work bound by HBM: one thread per ciphertext finds its
// length, a three-kernel exclusive scan places the items, and each warp
// writes 32 items (a lane per item for the headers, the whole warp on each
// payload with word stores).  Unpacking takes the item offsets (found by a
// host walk over the headers) and turns each item back into S limbs the same
// way round.
#include <cstdint>

#include "paillier_kernels.cuh"

namespace hg {

void count_launches(uint64_t n);

namespace {

constexpr int kWarpsPerBlock = 8;
constexpr int kScanBlock = 1024;

// Item k of the column-major DenseMatrix order (matrix.h:159-162) is element
// (k % rows, k / rows); in a row-major array that is (k % rows) * cols + k / rows.
// A vector or a single row is the same in both orders; otherwise the 32-bit
// division serves every matrix of fewer than 2^32 elements.
__device__ __forceinline__ size_t elem_of_item(size_t k, size_t rows, size_t cols, int row_major) {
  if (!row_major || rows == 1 || cols == 1) return k;
  if ((rows | k) >> 32) return (k % rows) * cols + k / rows;
  const uint32_t k32 = (uint32_t)k, r32 = (uint32_t)rows, q = k32 / r32;
  return (size_t)(k32 - q * r32) * cols + q;
}

__device__ __forceinline__ int bin_header_len(uint32_t b) { return b < 256u ? 2 : (b < 65536u ? 3 : 5); }
__device__ __forceinline__ int str_header_len(uint64_t l) {
  return l < 32u ? 1 : (l < 256u ? 2 : (l < 65536u ? 3 : 5));
}

// Per ciphertext (one thread each): magnitude bytes and the item's total
// bytes (str header included).  A full-size value has a nonzero top limb, so
// one 4-byte read usually decides.
__global__ void k_wire_sizes(const uint32_t* __restrict__ ct, size_t count, size_t rows, size_t cols, int row_major,
                             int S, uint32_t* __restrict__ mag_bytes, uint64_t* __restrict__ item_bytes) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const uint32_t* c = ct + elem_of_item(i, rows, cols, row_major) * (size_t)S;
  int top = S - 1;
  while (top >= 0 && c[top] == 0u) --top;
  const uint32_t b = top >= 0 ? (uint32_t)top * 4u + (uint32_t)((32 - __clz(c[top]) + 7) / 8) : 0u;
  const uint64_t inner = 1u + (uint64_t)bin_header_len(b) + b + 8u;  // fixarray(1), bin, schema
  mag_bytes[i] = b;
  item_bytes[i] = (uint64_t)str_header_len(inner) + inner;
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

// Each warp writes 32 consecutive items: every lane the headers and the
// schema trailer of its own item, then the warp copies the payloads one item
// after the other.
__global__ void k_wire_write(const uint32_t* __restrict__ ct, size_t count, size_t rows, size_t cols, int row_major,
                             int S, const uint32_t* __restrict__ mag_bytes, const uint64_t* __restrict__ offs,
                             const uint64_t* __restrict__ bsum, uint64_t schema, uint8_t* __restrict__ out,
                             size_t base, int aligned16) {
  const int lane = threadIdx.x & 31;
  const size_t first = ((size_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5)) * 32;
  if (first >= count) return;
  const size_t i = first + lane;
  uint32_t b = 0;
  uint64_t mpos = 0;  // payload position in out
  uint64_t e = 0;     // element index in ct
  if (i < count) {
    b = mag_bytes[i];
    const uint64_t inner = 1u + (uint64_t)bin_header_len(b) + b + 8u;
    const int sh = str_header_len(inner), bh = bin_header_len(b);
    const uint64_t at = base + offs[i] + bsum[i / kScanBlock];
    uint8_t* p = out + at;
    if (sh == 1) {
      p[0] = (uint8_t)(0xa0u | (uint32_t)inner);
    } else {
      p[0] = sh == 2 ? 0xd9 : (sh == 3 ? 0xda : 0xdb);
      put_be(p + 1, inner, sh - 1);
    }
    p[sh] = 0x91;  // fixarray(1): MSGPACK_DEFINE(c_)
    p[sh + 1] = bh == 2 ? 0xc4 : (bh == 3 ? 0xc5 : 0xc6);
    put_be(p + sh + 2, b, bh - 1);
    mpos = at + (uint64_t)(sh + 1 + bh);
    uint8_t* tr = out + mpos + b;
#pragma unroll
    for (int k = 0; k < 8; ++k) tr[k] = (uint8_t)(schema >> (8 * k));
    e = elem_of_item(i, rows, cols, row_major);
  }
  // Payloads, four items at a time so that their loads are in flight
  // together: in each round lane L holds source words w0 .. w0 + 3
  // (w0 = 128 * round + 4L, one 16-byte load) and writes destination words
  // w0 .. w0 + 3, word w being source words w and w + 1 shifted by the
  // payload's misalignment (the next lane's first word, by shuffle; lane 31
  // loads it).  Head and tail bytes are stored singly.
  const int nitems = (int)min((size_t)32, count - first);
  constexpr int kItems = 4;
  for (int t0 = 0; t0 < nitems; t0 += kItems) {
    uint32_t bt[kItems];
    uint8_t* mt[kItems];
    const uint32_t* ctt[kItems];
#pragma unroll
    for (int u = 0; u < kItems; ++u) {
      const int t = (t0 + u) & 31;
      bt[u] = __shfl_sync(0xffffffffu, b, t);
      mt[u] = out + __shfl_sync(0xffffffffu, mpos, t);
      ctt[u] = ct + __shfl_sync(0xffffffffu, e, t) * (size_t)S;
      if (t0 + u >= nitems) bt[u] = 0u;  // nothing to copy
    }
    for (int w0base = 0; w0base < S; w0base += 128) {
      const int w0 = w0base + 4 * lane;
      uint4 v[kItems];
      uint32_t nx[kItems];
#pragma unroll
      for (int u = 0; u < kItems; ++u) {
        const bool need = bt[u] > 0u && w0 < S && 4u * (uint32_t)w0 < bt[u];
        if (!need)
          v[u] = make_uint4(0u, 0u, 0u, 0u);
        else if (aligned16)
          v[u] = *reinterpret_cast<const uint4*>(ctt[u] + w0);
        else
          v[u] = make_uint4(ctt[u][w0], ctt[u][w0 + 1], ctt[u][w0 + 2], ctt[u][w0 + 3]);
        nx[u] = (need && lane == 31 && w0 + 4 < S) ? ctt[u][w0 + 4] : 0u;
      }
#pragma unroll
      for (int u = 0; u < kItems; ++u) {
        const uint32_t down = __shfl_down_sync(0xffffffffu, v[u].x, 1);
        if (bt[u] == 0u) continue;
        const uint32_t hi4 = lane == 31 ? nx[u] : down;
        uint8_t* m = mt[u];
        const uint32_t head = min((uint32_t)((4u - ((uint32_t)(uintptr_t)m & 3u)) & 3u), bt[u]);
        const uint32_t nw = (bt[u] - head) >> 2, sh = 8u * (head & 3u);
        uint32_t* dw = reinterpret_cast<uint32_t*>(m + head);
        const uint32_t src[5] = {v[u].x, v[u].y, v[u].z, v[u].w, hi4};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const uint32_t w = (uint32_t)(w0 + j);
          if (w < nw) dw[w] = __funnelshift_r(src[j], src[j + 1], sh);
        }
        if (w0base == 0) {
          const uint8_t* s8 = reinterpret_cast<const uint8_t*>(ctt[u]);
          if (lane < (int)head) m[lane] = s8[lane];
          const uint32_t done = head + 4u * nw;
          if (lane < (int)(bt[u] - done)) m[done + lane] = s8[done + lane];
        }
      }
    }
  }
}

// Each warp reads 32 consecutive items: every lane checks the headers of its
// own item (bytes [offs[i], offs[i] + lens[i]) of buf), then the warp turns
// the payloads into S limbs one item after the other.
__global__ void k_wire_read(const uint8_t* __restrict__ buf, const uint64_t* __restrict__ offs,
                            const uint64_t* __restrict__ lens, size_t count, size_t rows, size_t cols, int row_major,
                            int S, uint64_t schema, uint32_t* __restrict__ out, uint32_t* err) {
  const int lane = threadIdx.x & 31;
  const size_t first = ((size_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5)) * 32;
  if (first >= count) return;
  const size_t i = first + lane;
  bool ok = false;
  uint64_t b = 0, mpos = 0, e = 0;
  if (i < count) {
    const uint8_t* p = buf + offs[i];
    const uint64_t len = lens[i];
    ok = len >= 1u + 2u + 8u && p[0] == 0x91;
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
    if (!ok) atomicOr(err, kErrFormat);
    mpos = offs[i] + 1u + (uint64_t)bh;
    e = elem_of_item(i, rows, cols, row_major);
  }
  const int nitems = (int)min((size_t)32, count - first);
  for (int t = 0; t < nitems; ++t) {
    const bool okt = __shfl_sync(0xffffffffu, ok, t);
    const uint64_t bt = __shfl_sync(0xffffffffu, b, t);
    const uint64_t mt = __shfl_sync(0xffffffffu, mpos, t);
    const uint64_t et = __shfl_sync(0xffffffffu, e, t);
    uint32_t* o = out + et * (size_t)S;
    if (!okt) {
      for (int j = lane; j < S; j += 32) o[j] = 0u;
      continue;
    }
    // limb j = bytes [4j, 4j + 4) of the magnitude (zero past bt): whole limbs
    // from the aligned words around them, the last partial limb bytewise
    const uint8_t* m = buf + mt;
    const uint32_t mis = (uint32_t)(uintptr_t)m & 3u;
    const uint32_t* aw = reinterpret_cast<const uint32_t*>(m - mis);
    const uint32_t full = (uint32_t)(bt >> 2);
    for (int j = lane; j < S; j += 32) {
      uint32_t v = 0u;
      if ((uint32_t)j < full) {
        const uint32_t lo = aw[j], hi = mis ? aw[j + 1] : 0u;  // aw[j + 1] holds bytes < 4j + 4 + mis <= bt + 3
        v = __funnelshift_r(lo, hi, 8u * mis);
      } else {
        for (int k = 3; k >= 0; --k) {
          const uint64_t at = 4u * (uint64_t)j + (uint64_t)k;
          v = (v << 8) | (at < bt ? m[at] : 0u);
        }
      }
      o[j] = v;
    }
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
  const unsigned gs = (unsigned)((count + 255) / 256);
  k_wire_sizes<<<gs, 256, 0, st>>>(ct, count, rows, cols, row_major, S, mag_bytes, items);
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
  const unsigned g = (unsigned)((count + 32 * kWarpsPerBlock - 1) / (32 * kWarpsPerBlock));
  // 16-byte loads need a 16-byte aligned ct (rows are S * 4 = 256 / 512 / 768 bytes)
  const int aligned16 = ((uintptr_t)ct & 15u) == 0 && (S * 4) % 16 == 0;
  k_wire_write<<<g, 32 * kWarpsPerBlock, 0, st>>>(ct, count, rows, cols, row_major, S, mag_bytes, scratch,
                                                   scratch + count, schema, out, base, aligned16);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_wire_unpack(const uint8_t* buf, const uint64_t* offs, const uint64_t* lens, size_t rows,
                               size_t cols, int row_major, int S, uint64_t schema, uint32_t* out, uint32_t* err,
                               cudaStream_t st) {
  const size_t count = rows * cols;
  if (count == 0) return cudaSuccess;
  const unsigned g = (unsigned)((count + 32 * kWarpsPerBlock - 1) / (32 * kWarpsPerBlock));
  k_wire_read<<<g, 32 * kWarpsPerBlock, 0, st>>>(buf, offs, lens, count, rows, cols, row_major, S, schema, out, err);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace hg

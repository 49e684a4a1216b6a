// heu.numpy MatMul of a ciphertext matrix by an integer plaintext matrix
// (numpy/evaluator.cc:208-292): out(i,j) = prod_k x(i,k)^y(k,j) mod n^2.
//
// The bases x(i,.) of one row are shared by every output column, so the row
// is cut into chunks of 8 bases and each chunk gets the table of all 256
// subset products (247 multiplications).  With the exponents shifted to
// y' = y + o >= 0 (o = -min y when y has negatives) and written in P bit
// planes, every output is a Horner pass over the planes:
//   acc = acc^2; acc *= prod_chunks table[chunk][bits of y'(chunk, j) in plane]
// and the shift is undone with (prod_k x(i,k))^-o, one inverse per row.
#include <algorithm>

#include "mont.cuh"
#include "paillier_kernels.cuh"

namespace hg {

namespace {
constexpr int kBlock = 128;
constexpr int kChunk = 8;
constexpr int kSubsets = 1 << kChunk;
}  // namespace

// T[(i * nch + c) * 256 + mask] = prod_{b in mask} x(r0 + i, 8c + b), mask 0 = R
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_subset_tables(KeyConst kc, const uint32_t* __restrict__ x, size_t r0,
                                                          size_t rows, int K, int nch, uint32_t* __restrict__ T,
                                                          uint32_t* err) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  const size_t total = rows * (size_t)nch;
  if (wfirst >= total) return;
  const bool active = inst < total;
  const size_t u = active ? inst : total - 1;
  const size_t i = u / nch;
  const int c = (int)(u % nch);
  uint32_t N[L], a[L], b[L];
  load_slice<L>(N, kc.N + g.t * L);
  uint32_t* tab = T + u * kSubsets * S + g.t * L;
  load_slice<L>(a, kc.R1 + g.t * L);
  if (active) store_slice<L>(tab, a);
  const uint32_t* xrow = x + ((r0 + i) * (size_t)K) * S;
#pragma unroll 1
  for (int bit = 0; bit < kChunk; ++bit) {
    const int k = c * kChunk + bit;
    load_slice<L>(a, (k < K ? xrow + (size_t)k * S : kc.R1) + g.t * L);
    uint32_t d[L];
    const bool bad = sub_full<TPI, L>(d, a, N, g) == 0u;
    if (active && k < K && bad && g.t == 0) atomicOr(err, kErrCtRange);
    if (active) store_slice<L>(tab + (size_t)(1 << bit) * S, a);
  }
  // masks with two or more bits: T[mask] = T[mask without its top bit] * T[top bit]
#pragma unroll 1
  for (int top = 1; top < kChunk; ++top) {
    load_slice<L>(b, tab + (size_t)(1 << top) * S);
#pragma unroll 1
    for (int rest = 1; rest < (1 << top); ++rest) {
      load_slice<L>(a, tab + (size_t)rest * S);
      mont_mul<TPI, L>(a, a, b, N, kc.np, g);
      if (active) store_slice<L>(tab + (size_t)((1 << top) | rest) * S, a);
    }
  }
}

// out(r0 + i, j) = prod over planes (Horner) of table products selected by masks
// masks[(j * P + plane) * nch + c] = bits of y'(8c .. 8c+7, j) in `plane`
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_matmul_planes(KeyConst kc, const uint32_t* __restrict__ T,
                                                          const uint8_t* __restrict__ masks, size_t r0, size_t rows,
                                                          int Ncols, int P, int nch, uint32_t* __restrict__ out) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  const size_t total = rows * (size_t)Ncols;
  if (wfirst >= total) return;
  const bool active = inst < total;
  const size_t u = active ? inst : total - 1;
  const size_t i = u / Ncols;
  const int j = (int)(u % Ncols);
  uint32_t N[L], acc[L], b[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(acc, kc.R1 + g.t * L);
  const uint32_t* tab = T + (i * nch) * (size_t)kSubsets * S + g.t * L;
#pragma unroll 1
  for (int plane = P - 1; plane >= 0; --plane) {
    if (plane != P - 1) mont_mul<TPI, L>(acc, acc, acc, N, kc.np, g);
    const uint8_t* mk = masks + ((size_t)j * P + plane) * nch;
#pragma unroll 1
    for (int c = 0; c < nch; ++c) {
      const uint32_t m = mk[c];
      load_slice<L>(b, tab + ((size_t)c * kSubsets + m) * S);
      mont_mul<TPI, L>(acc, acc, b, N, kc.np, g);
    }
  }
  if (active) store_slice<L>(out + ((r0 + i) * (size_t)Ncols + j) * S + g.t * L, acc);
}

// prod[i] = prod_k x(r0 + i, k), read from the full-mask entries of the tables
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_row_products(KeyConst kc, const uint32_t* __restrict__ T, size_t rows,
                                                         int K, int nch, uint32_t* __restrict__ prod) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  if (wfirst >= rows) return;
  const bool active = inst < rows;
  const size_t i = active ? inst : rows - 1;
  uint32_t N[L], acc[L], b[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(acc, kc.R1 + g.t * L);
#pragma unroll 1
  for (int c = 0; c < nch; ++c) {
    const int nb = min(kChunk, K - c * kChunk);
    const size_t full = (size_t)((1 << nb) - 1);
    load_slice<L>(b, T + ((i * nch + c) * kSubsets + full) * S + g.t * L);
    mont_mul<TPI, L>(acc, acc, b, N, kc.np, g);
  }
  if (active) store_slice<L>(prod + i * S + g.t * L, acc);
}

// v[i] = v[i]^e for one 64-bit exponent e >= 1 shared by all instances
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_pow_shared(KeyConst kc, uint32_t* __restrict__ v, size_t count,
                                                       uint64_t e) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  if (wfirst >= count) return;
  const bool active = inst < count;
  const size_t i = active ? inst : count - 1;
  uint32_t N[L], x[L], acc[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(x, v + i * S + g.t * L);
  copy_slice<L>(acc, x);
  const int top = 63 - __clzll((long long)e);
#pragma unroll 1
  for (int bit = top - 1; bit >= 0; --bit) {
    mont_mul<TPI, L>(acc, acc, acc, N, kc.np, g);
    if ((e >> bit) & 1ull) mont_mul<TPI, L>(acc, acc, x, N, kc.np, g);
  }
  if (active) store_slice<L>(v + i * S + g.t * L, acc);
}

// v[i] = v[i]^e for one multi-limb exponent e >= 1 (el limbs, device memory)
// shared by all instances: left-to-right square-and-multiply
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_pow_shared_bn(KeyConst kc, uint32_t* __restrict__ v, size_t count,
                                                          const uint32_t* __restrict__ e, int el) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  if (wfirst >= count) return;
  const bool active = inst < count;
  const size_t i = active ? inst : count - 1;
  int top = -1;
#pragma unroll 1
  for (int l = el - 1; l >= 0 && top < 0; --l)
    if (e[l] != 0u) top = l * 32 + 31 - __clz(e[l]);
  if (top < 0) return;  // e = 0 is not passed by the host
  uint32_t N[L], x[L], acc[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(x, v + i * S + g.t * L);
  copy_slice<L>(acc, x);
#pragma unroll 1
  for (int bit = top - 1; bit >= 0; --bit) {
    mont_mul<TPI, L>(acc, acc, acc, N, kc.np, g);
    if ((e[bit >> 5] >> (bit & 31)) & 1u) mont_mul<TPI, L>(acc, acc, x, N, kc.np, g);
  }
  if (active) store_slice<L>(v + i * S + g.t * L, acc);
}

// out(r0 + i, j) *= q[i]
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_scale_rows(KeyConst kc, uint32_t* __restrict__ out,
                                                       const uint32_t* __restrict__ q, size_t r0, size_t rows,
                                                       int Ncols) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  const size_t total = rows * (size_t)Ncols;
  if (wfirst >= total) return;
  const bool active = inst < total;
  const size_t u = active ? inst : total - 1;
  const size_t i = u / Ncols;
  uint32_t N[L], a[L], b[L];
  load_slice<L>(N, kc.N + g.t * L);
  uint32_t* p = out + (r0 * Ncols + u) * S + g.t * L;
  load_slice<L>(a, p);
  load_slice<L>(b, q + i * S + g.t * L);
  mont_mul<TPI, L>(a, a, b, N, kc.np, g);
  if (active) store_slice<L>(p, a);
}

#define HG_DISPATCH_S3(S, ...)                                          \
  switch (S) {                                                          \
    case 64: { constexpr int TPI = 4, L = 16; __VA_ARGS__; } break;     \
    case 128: { constexpr int TPI = 8, L = 16; __VA_ARGS__; } break;    \
    case 192: { constexpr int TPI = 16, L = 12; __VA_ARGS__; } break;   \
    default: return cudaErrorInvalidValue;                              \
  }

static inline unsigned nblocks(size_t inst, int tpi) {
  const size_t ipb = kBlock / tpi;
  return (unsigned)((inst + ipb - 1) / ipb);
}

cudaError_t launch_subset_tables(int S, const KeyConst& kc, const uint32_t* x, size_t r0, size_t rows, int K,
                                 uint32_t* T, uint32_t* err, cudaStream_t st) {
  const int nch = (K + kChunk - 1) / kChunk;
  HG_DISPATCH_S3(S, k_subset_tables<TPI, L><<<nblocks(rows * nch, TPI), kBlock, 0, st>>>(kc, x, r0, rows, K, nch, T,
                                                                                        err));
  return cudaGetLastError();
}

cudaError_t launch_matmul_planes(int S, const KeyConst& kc, const uint32_t* T, const uint8_t* masks, size_t r0,
                                 size_t rows, int Ncols, int P, int K, uint32_t* out, cudaStream_t st) {
  const int nch = (K + kChunk - 1) / kChunk;
  HG_DISPATCH_S3(S, k_matmul_planes<TPI, L><<<nblocks(rows * Ncols, TPI), kBlock, 0, st>>>(kc, T, masks, r0, rows,
                                                                                          Ncols, P, nch, out));
  return cudaGetLastError();
}

cudaError_t launch_row_products(int S, const KeyConst& kc, const uint32_t* T, size_t rows, int K, uint32_t* prod,
                                cudaStream_t st) {
  const int nch = (K + kChunk - 1) / kChunk;
  HG_DISPATCH_S3(S, k_row_products<TPI, L><<<nblocks(rows, TPI), kBlock, 0, st>>>(kc, T, rows, K, nch, prod));
  return cudaGetLastError();
}

cudaError_t launch_pow_shared(int S, const KeyConst& kc, uint32_t* v, size_t count, uint64_t e, cudaStream_t st) {
  if (e <= 1) return cudaSuccess;
  HG_DISPATCH_S3(S, k_pow_shared<TPI, L><<<nblocks(count, TPI), kBlock, 0, st>>>(kc, v, count, e));
  return cudaGetLastError();
}

cudaError_t launch_pow_shared_bn(int S, const KeyConst& kc, uint32_t* v, size_t count, const uint32_t* e, int el,
                                 cudaStream_t st) {
  if (count == 0 || el < 1) return cudaSuccess;
  HG_DISPATCH_S3(S, k_pow_shared_bn<TPI, L><<<nblocks(count, TPI), kBlock, 0, st>>>(kc, v, count, e, el));
  return cudaGetLastError();
}

cudaError_t launch_scale_rows(int S, const KeyConst& kc, uint32_t* out, const uint32_t* q, size_t r0, size_t rows,
                              int Ncols, cudaStream_t st) {
  HG_DISPATCH_S3(S, k_scale_rows<TPI, L><<<nblocks(rows * Ncols, TPI), kBlock, 0, st>>>(kc, out, q, r0, rows,
                                                                                       Ncols));
  return cudaGetLastError();
}

size_t subset_table_bytes_per_row(int S, int K) {
  const int nch = (K + kChunk - 1) / kChunk;
  return (size_t)nch * kSubsets * S * 4;
}

}  // namespace hg

// Paillier (DJN variant, HEU paillier_z semantics) kernels for sm_103a.
//
// Every ciphertext is handled by a group of TPI lanes (mont.cuh); the
// per-ciphertext bodies live in paillier_ops.cuh.  The kernels keep warps
// converged: loop trip counts are uniform per warp, tails compute on a
// clamped index and skip their stores, and per-instance choices (square vs
// multiply, which table entry) only change the data a uniform Montgomery
// multiplication consumes.
#include <algorithm>
#include <atomic>

#include "paillier_ops.cuh"

namespace hg {

constexpr int kBlock = 128;  // threads per block for every kernel here

#define HG_INSTANCE_PROLOGUE(COUNT)                                                      \
  const Group<TPI> g;                                                                    \
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;                \
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;     \
  if (wfirst >= (COUNT)) return;                                                         \
  const bool active = inst < (COUNT);                                                    \
  const size_t i = active ? inst : (COUNT)-1;

template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_encrypt(KeyConst kc, EncMode mode, const int64_t* __restrict__ m,
                                                    const uint32_t* __restrict__ m_mag,
                                                    const uint8_t* __restrict__ m_neg,
                                                    const uint32_t* __restrict__ r,
                                                    const uint32_t* __restrict__ ct_in, uint32_t* __restrict__ out,
                                                    size_t count, uint32_t* err, Codec cd) {
  HG_INSTANCE_PROLOGUE(count)
  uint32_t N[L];
  load_slice<L>(N, kc.N + g.t * L);
  encrypt_one<TPI, L>(kc, mode, m, m_mag, m_neg, r, ct_in, out, i, active, N, g, err, cd);
}

template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_add(KeyConst kc, const uint32_t* __restrict__ a,
                                                const uint32_t* __restrict__ b, uint32_t* __restrict__ out,
                                                size_t count, uint32_t* err) {
  HG_INSTANCE_PROLOGUE(count)
  uint32_t N[L];
  load_slice<L>(N, kc.N + g.t * L);
  add_one<TPI, L>(kc, a, b, out, i, active, N, g, err);
}

template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_add_plain(KeyConst kc, const uint32_t* __restrict__ a,
                                                      const int64_t* __restrict__ p, int neg_p,
                                                      uint32_t* __restrict__ out, size_t count, uint32_t* err) {
  HG_INSTANCE_PROLOGUE(count)
  uint32_t N[L];
  load_slice<L>(N, kc.N + g.t * L);
  add_plain_one<TPI, L>(kc, a, p, neg_p, out, i, active, N, g, err);
}

template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_convert(KeyConst kc, const uint32_t* __restrict__ in,
                                                    uint32_t* __restrict__ out, size_t count, int to_mont,
                                                    uint32_t* err) {
  HG_INSTANCE_PROLOGUE(count)
  uint32_t N[L];
  load_slice<L>(N, kc.N + g.t * L);
  convert_one<TPI, L>(kc, in, out, to_mont, i, active, N, g, err);
}

// out = MM(in, C) = in * C * R^-1 for one constant C (device memory): moves
// Montgomery residues between radices (C = R_ext mod N to the radix R_ext,
// R^2 * R_ext^-1 mod N back).
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_mul_const(KeyConst kc, const uint32_t* __restrict__ in,
                                                      const uint32_t* __restrict__ c, uint32_t* __restrict__ out,
                                                      size_t count, uint32_t* err) {
  constexpr int S = TPI * L;
  HG_INSTANCE_PROLOGUE(count)
  uint32_t N[L], A[L], B[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(A, in + i * S + g.t * L);
  check_ct<TPI, L>(A, N, active, g, err);
  load_slice<L>(B, c + g.t * L);
  mont_mul<TPI, L>(A, A, B, N, kc.np, g);
  if (active) store_slice<L>(out + i * S + g.t * L, A);
}

// Persistent: each instance slot of the grid owns an odd-power table.
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_mul(KeyConst kc, const uint32_t* __restrict__ a,
                                                const int64_t* __restrict__ kk, uint32_t* __restrict__ out,
                                                size_t count, uint32_t* __restrict__ scratch, int wm,
                                                uint32_t* err, unsigned long long* ctr) {
  constexpr int S = TPI * L;
  constexpr int IPB = kBlock / TPI;
  constexpr int IPW = 32 / TPI;
  const Group<TPI> g;
  const int lane_inst = (threadIdx.x & 31) / TPI;
  const int warp_first = (threadIdx.x >> 5) * IPW;
  const int ntab = 1 << (wm - 1);
  uint32_t* tb = scratch + ((size_t)blockIdx.x * IPB + warp_first + lane_inst) * (size_t)ntab * S + g.t * L;
  uint32_t N[L];
  load_slice<L>(N, kc.N + g.t * L);
  for (size_t wbase = next_work(ctr, IPW); wbase < count; wbase = next_work(ctr, IPW)) {
    const size_t inst = wbase + lane_inst;
    const bool active = inst < count;
    mul_one<TPI, L>(kc, a, kk, out, active ? inst : count - 1, active, tb, wm, N, g, err);
  }
}

// Mul by multi-limb scalars; persistent like k_mul (one odd-power table of
// 2^(wb-1) entries per instance slot of the grid).
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_mul_bn(KeyConst kc, const uint32_t* __restrict__ a,
                                                   const uint32_t* __restrict__ emag, int el,
                                                   uint32_t* __restrict__ out, size_t count,
                                                   uint32_t* __restrict__ scratch, int wb, uint32_t* err,
                                                   unsigned long long* ctr) {
  constexpr int S = TPI * L;
  constexpr int IPB = kBlock / TPI;
  constexpr int IPW = 32 / TPI;
  const Group<TPI> g;
  const int lane_inst = (threadIdx.x & 31) / TPI;
  const int warp_first = (threadIdx.x >> 5) * IPW;
  const int ntab = 1 << (wb - 1);
  uint32_t* tb = scratch + ((size_t)blockIdx.x * IPB + warp_first + lane_inst) * (size_t)ntab * S + g.t * L;
  uint32_t N[L];
  load_slice<L>(N, kc.N + g.t * L);
  for (size_t wbase = next_work(ctr, IPW); wbase < count; wbase = next_work(ctr, IPW)) {
    const size_t inst = wbase + lane_inst;
    const bool active = inst < count;
    mul_bn_one<TPI, L>(kc, a, emag, el, out, active ? inst : count - 1, active, tb, wb, N, g, err);
  }
}

// sel[i] = -1 where neg[i] != 0, else 1 (the inverse's selector)
__global__ void k_sel_from_neg(const uint8_t* __restrict__ neg, int64_t* __restrict__ sel, size_t count) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) sel[i] = neg[i] ? -1 : 1;
}

// Chunked product reduction: out[j] = prod in[j*chunk .. (j+1)*chunk)
// (numpy/evaluator.cc:355-373 reduces with AddInplace = MulMod)
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_reduce(KeyConst kc, const uint32_t* __restrict__ in, size_t count,
                                                   int chunk, uint32_t* __restrict__ out, size_t out_count,
                                                   uint32_t* err) {
  constexpr int S = TPI * L;
  HG_INSTANCE_PROLOGUE(out_count)
  uint32_t N[L], acc[L];
  load_slice<L>(N, kc.N + g.t * L);
  const size_t first = i * (size_t)chunk;
  load_slice<L>(acc, in + first * S + g.t * L);
  check_ct<TPI, L>(acc, N, active, g, err);
#pragma unroll 1
  for (int j = 1; j < chunk; ++j) {
    const size_t idx = first + j;
    const bool valid = idx < count;
    if (!__any_sync(kFull, valid)) break;
    uint32_t B[L];
    load_slice<L>(B, (valid ? in + idx * S : kc.R1) + g.t * L);
    // every input is range-checked before it enters mont_mul (b < N)
    check_ct<TPI, L>(B, N, active && valid, g, err);
    mont_mul<TPI, L>(acc, acc, B, N, kc.np, g);
  }
  if (active) store_slice<L>(out + i * S + g.t * L, acc);
}

// Sum as a tree of modular products (numpy/evaluator.cc:355-373 reduces with
// AddInplace = MulMod): each group of TPI lanes multiplies its chunk of
// `chunk` inputs in sequence (every input range-checked), then the groups of
// a warp combine pairwise through shuffles (log2(32/TPI) levels, one
// Montgomery multiplication each), and warp 0 multiplies in the other warps'
// products from shared memory: one ciphertext per block, out[blockIdx.x].
// Missing inputs count as the identity R.
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_reduce_tree(KeyConst kc, const uint32_t* __restrict__ in, size_t count,
                                                        int chunk, uint32_t* __restrict__ out, uint32_t* err) {
  constexpr int S = TPI * L;
  constexpr int IPW = 32 / TPI;
  constexpr int kWarps = kBlock / 32;
  __shared__ __align__(16) uint32_t wsum[kWarps][S];
  const Group<TPI> g;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  uint32_t N[L], acc[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(acc, kc.R1 + g.t * L);
  const size_t first = inst * (size_t)chunk;
#pragma unroll 1
  for (int j = 0; j < chunk; ++j) {
    const size_t idx = first + j;
    const bool valid = idx < count;
    if (!__any_sync(kFull, valid)) break;
    uint32_t B[L];
    load_slice<L>(B, (valid ? in + idx * S : kc.R1) + g.t * L);
    check_ct<TPI, L>(B, N, valid, g, err);
    if (j == 0) {
      // the first input starts the product (acc is R, the identity)
#pragma unroll
      for (int t = 0; t < L; ++t) acc[t] = B[t];
    } else {
      mont_mul<TPI, L>(acc, acc, B, N, kc.np, g);
    }
  }
  // groups of the warp: group k takes group k + d's product (k % 2d == 0)
#pragma unroll
  for (int d = 1; d < IPW; d <<= 1) {
    uint32_t B[L];
#pragma unroll
    for (int j = 0; j < L; ++j) B[j] = __shfl_down_sync(kFull, acc[j], d * TPI);
    const bool take = ((lane / TPI) % (2 * d) == 0) && (lane / TPI + d < IPW);
    if (!take) load_slice<L>(B, kc.R1 + g.t * L);
    mont_mul<TPI, L>(acc, acc, B, N, kc.np, g);
  }
  // warps of the block, as a tree through shared memory: warp w takes warp
  // w + d's product (w % 2d == 0); warp 0 ends with the block's product
  if (lane < TPI) store_slice<L>(&wsum[warp][g.t * L], acc);
  __syncthreads();
#pragma unroll
  for (int d = 1; d < kWarps; d <<= 1) {
    if (warp % (2 * d) == 0 && warp + d < kWarps) {
      uint32_t B[L];
      load_slice<L>(B, &wsum[warp + d][g.t * L]);
      mont_mul<TPI, L>(acc, acc, B, N, kc.np, g);
      if (lane < TPI) store_slice<L>(&wsum[warp][g.t * L], acc);
    }
    __syncthreads();
  }
  if (warp == 0 && lane < TPI) store_slice<L>(out + (size_t)blockIdx.x * S + g.t * L, acc);
}

// ---------------------------------------------------------------------------
// Product tree for batch inversion (Montgomery's simultaneous-inversion
// trick arranged as a tree): leaves, up-sweep, root fix, down-sweep, apply.
// ---------------------------------------------------------------------------
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_tree_leaves(KeyConst kc, const uint32_t* __restrict__ in,
                                                        const int64_t* __restrict__ sel, size_t count,
                                                        uint32_t* __restrict__ leaves, size_t padded,
                                                        uint32_t* err) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  if (wfirst >= padded) return;
  const size_t i = inst < count ? inst : count - 1;
  uint32_t A[L], N[L], one[L];
  load_slice<L>(A, in + i * S + g.t * L);
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(one, kc.R1 + g.t * L);
  const bool use = inst < count && (sel == nullptr || sel[i] < 0);
  check_ct<TPI, L>(A, N, use, g, err);
  select_slice<L>(A, use, A, one);
  if (inst < padded) store_slice<L>(leaves + inst * S + g.t * L, A);
}

template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_tree_up(KeyConst kc, const uint32_t* __restrict__ lower,
                                                    uint32_t* __restrict__ upper, size_t upper_count) {
  constexpr int S = TPI * L;
  HG_INSTANCE_PROLOGUE(upper_count)
  uint32_t N[L], A[L], B[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(A, lower + (2 * i) * S + g.t * L);
  load_slice<L>(B, lower + (2 * i + 1) * S + g.t * L);
  mont_mul<TPI, L>(A, A, B, N, kc.np, g);
  if (active) store_slice<L>(upper + i * S + g.t * L, A);
}

template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_tree_down(KeyConst kc, uint32_t* __restrict__ lower,
                                                      const uint32_t* __restrict__ upper_inv, size_t upper_count) {
  constexpr int S = TPI * L;
  HG_INSTANCE_PROLOGUE(upper_count)
  uint32_t N[L], U[L], A[L], B[L], ra[L], rb[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(U, upper_inv + i * S + g.t * L);
  load_slice<L>(A, lower + (2 * i) * S + g.t * L);
  load_slice<L>(B, lower + (2 * i + 1) * S + g.t * L);
  mont_mul<TPI, L>(ra, U, B, N, kc.np, g);  // inverse of A
  mont_mul<TPI, L>(rb, U, A, N, kc.np, g);  // inverse of B
  if (active) {
    store_slice<L>(lower + (2 * i) * S + g.t * L, ra);
    store_slice<L>(lower + (2 * i + 1) * S + g.t * L, rb);
  }
}

template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_tree_apply(KeyConst kc, const uint32_t* __restrict__ in,
                                                       const int64_t* __restrict__ sel,
                                                       const uint32_t* __restrict__ leaves_inv,
                                                       uint32_t* __restrict__ out, size_t count) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  if (inst >= count) return;
  uint32_t A[L];
  const bool use = (sel == nullptr || sel[inst] < 0);
  load_slice<L>(A, (use ? leaves_inv : in) + inst * S + g.t * L);
  store_slice<L>(out + inst * S + g.t * L, A);
}

// ---------------------------------------------------------------------------
// Fixed-base table (public_key.cc:28-40 builds yacl's BaseTable on the host):
//   bases[pos] = h_s^(2^(w*pos)) (one group, sequential squarings)
//   table[pos][d-1] = bases[pos]^d for d in [1, 2^w)
// ---------------------------------------------------------------------------
template <int TPI, int L>
__global__ void __launch_bounds__(32) k_table_bases(KeyConst kc, const uint32_t* __restrict__ hs_mont,
                                                    uint32_t* __restrict__ bases) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  uint32_t N[L], x[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(x, hs_mont + g.t * L);
  for (int pos = 0; pos < kc.npos; ++pos) {
    if (threadIdx.x < TPI) store_slice<L>(bases + (size_t)pos * S + g.t * L, x);
#pragma unroll 1
    for (int s = 0; s < kc.w; ++s) mont_mul<TPI, L>(x, x, x, N, kc.np, g);
  }
}

// level < 0: copy bases into entry d = 1; level j >= 0: entries
// d in [2^j + 1, min(2^(j+1), 2^w - 1)] = entry(2^j) * entry(d - 2^j).
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_table_level(KeyConst kc, uint32_t* __restrict__ table,
                                                        const uint32_t* __restrict__ bases, int level) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t ent = (size_t)((1u << kc.w) - 1u);
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  if (level < 0) {
    if (inst >= (size_t)kc.npos) return;
    uint32_t A[L];
    load_slice<L>(A, bases + inst * S + g.t * L);
    store_slice<L>(table + inst * ent * S + g.t * L, A);
    return;
  }
  const size_t lo = (1ull << level) + 1ull;
  const size_t hi = min((size_t)(1ull << (level + 1)), ent);
  if (hi < lo) return;
  const size_t per = hi - lo + 1;
  const size_t total = per * (size_t)kc.npos;
  if (wfirst >= total) return;
  const bool active = inst < total;
  const size_t k = active ? inst : total - 1;
  const size_t pos = k / per, d = lo + k % per;
  uint32_t N[L], A[L], B[L];
  load_slice<L>(N, kc.N + g.t * L);
  const uint32_t* row = table + pos * ent * S;
  load_slice<L>(A, row + ((1ull << level) - 1ull) * S + g.t * L);
  load_slice<L>(B, row + (d - (1ull << level) - 1ull) * S + g.t * L);
  mont_mul<TPI, L>(A, A, B, N, kc.np, g);
  if (active) store_slice<L>(table + (pos * ent + d - 1) * S + g.t * L, A);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
bool supported_limbs(int S) { return S == 64 || S == 128 || S == 192; }

static std::atomic<uint64_t> g_launches{0};
uint64_t launch_count() { return g_launches.load(); }
void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
static inline cudaError_t counted() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaGetLastError();
}

static inline unsigned blocks_for(size_t instances, int tpi) {
  const size_t ipb = kBlock / tpi;
  return (unsigned)((instances + ipb - 1) / ipb);
}

template <typename K>
static int occupancy_blocks(K kernel, size_t smem = 0) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kBlock, smem);
  return sms * (per > 0 ? per : 1);
}

int instances_per_block(int S, int variant) {
  const int tpi = (S == 64) ? (variant ? 8 : 4) : (S == 128) ? (variant ? 4 : 8) : (variant ? 8 : 16);
  return kBlock / tpi;
}

// Batches up to this size run in the latency layout (one instance per
// warp): they leave the GPU mostly idle in the throughput layout and finish
// sooner with fewer limbs per lane on each dependent chain.  The bound is
// one wave of the latency layout, and at most 12 instances per SM: beyond
// that the latency layout's lower efficiency per multiplication (more
// shuffles per limb) costs more than its shorter chains save (measured on
// GB300: 4096 encryptions took 1.66 ms in the latency layout against
// 1.47 ms in the throughput layout, one took 0.38 ms against 0.91 ms).
template <typename K>
static size_t latency_wave(K kernel) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return std::min((size_t)occupancy_blocks(kernel) * (kBlock / 32), (size_t)12 * (size_t)sms);
}

static size_t latency_wave_encrypt(int S) {
  static size_t cache[3] = {0, 0, 0};
  const int slot = S == 64 ? 0 : S == 128 ? 1 : 2;
  if (cache[slot] == 0) {
    size_t v = 0;
    [&]() -> cudaError_t { HG_DISPATCH_SL(S, v = latency_wave(k_encrypt<TPI, L>)); return cudaSuccess; }();
    cache[slot] = v;
  }
  return cache[slot];
}

static size_t latency_wave_mul(int S) {
  static size_t cache[3] = {0, 0, 0};
  const int slot = S == 64 ? 0 : S == 128 ? 1 : 2;
  if (cache[slot] == 0) {
    size_t v = 0;
    [&]() -> cudaError_t { HG_DISPATCH_SL(S, v = latency_wave(k_mul<TPI, L>)); return cudaSuccess; }();
    cache[slot] = v;
  }
  return cache[slot];
}

int resident_blocks_mul(int S, int variant) {
  int r = 0;
  [&]() -> cudaError_t { HG_DISPATCH_SV(S, variant, r = occupancy_blocks(k_mul<TPI, L>)); return cudaSuccess; }();
  return r;
}

cudaError_t launch_encrypt(int S, const KeyConst& kc, EncMode mode, const int64_t* m, const uint32_t* m_mag,
                           const uint8_t* m_neg, const uint32_t* r, const uint32_t* ct_in, uint32_t* out,
                           size_t count, uint32_t* err, int grid, cudaStream_t st, const Codec& cd) {
  (void)grid;
  if (count == 0) return cudaSuccess;
  if (count <= latency_wave_encrypt(S)) {
    HG_DISPATCH_SL(S, k_encrypt<TPI, L><<<blocks_for(count, TPI), kBlock, 0, st>>>(kc, mode, m, m_mag, m_neg, r,
                                                                                  ct_in, out, count, err, cd));
    return counted();
  }
  HG_DISPATCH_SV(S, kc.variant,
                 k_encrypt<TPI, L><<<blocks_for(count, TPI), kBlock, 0, st>>>(kc, mode, m, m_mag, m_neg, r, ct_in,
                                                                             out, count, err, cd));
  return counted();
}

cudaError_t launch_add(int S, const KeyConst& kc, const uint32_t* a, const uint32_t* b, uint32_t* out,
                       size_t count, uint32_t* err, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  HG_DISPATCH_S0(S,
                 k_add<TPI, L><<<blocks_for(count, TPI), kBlock, 0, st>>>(kc, a, b, out, count, err));
  return counted();
}

cudaError_t launch_add_plain(int S, const KeyConst& kc, const uint32_t* a, const int64_t* p, int neg_p,
                             uint32_t* out, size_t count, uint32_t* err, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  HG_DISPATCH_S0(S,
                 k_add_plain<TPI, L><<<blocks_for(count, TPI), kBlock, 0, st>>>(kc, a, p, neg_p, out, count, err));
  return counted();
}

cudaError_t launch_mul(int S, const KeyConst& kc, const uint32_t* a, const int64_t* k, uint32_t* out,
                       size_t count, uint32_t* scratch, int wm, uint32_t* err, int grid, unsigned long long* ctr,
                       cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  const cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(*ctr), st);
  if (e != cudaSuccess) return e;
  // the latency layout's instance slots must fit the scratch sized for
  // `grid` blocks of the throughput layout
  const size_t lat_blocks = blocks_for(count, 32);
  if (count <= latency_wave_mul(S) &&
      lat_blocks * (kBlock / 32) <= (size_t)grid * instances_per_block(S, kc.variant)) {
    HG_DISPATCH_SL(S, k_mul<TPI, L><<<(unsigned)lat_blocks, kBlock, 0, st>>>(kc, a, k, out, count, scratch, wm, err,
                                                                            ctr));
    return counted();
  }
  HG_DISPATCH_SV(S, kc.variant, {
    const unsigned need = blocks_for(count, TPI);
    const unsigned gb = (unsigned)std::min((size_t)need, (size_t)grid);
    k_mul<TPI, L><<<gb, kBlock, 0, st>>>(kc, a, k, out, count, scratch, wm, err, ctr);
  });
  return counted();
}

cudaError_t launch_mul_bn(int S, const KeyConst& kc, const uint32_t* a, const uint32_t* emag, int el,
                          uint32_t* out, size_t count, uint32_t* scratch, int wb, uint32_t* err, int grid,
                          unsigned long long* ctr, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  if (el < 1 || wb < 1 || wb > 8) return cudaErrorInvalidValue;
  const cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(*ctr), st);
  if (e != cudaSuccess) return e;
  HG_DISPATCH_S0(S, {
    const unsigned need = blocks_for(count, TPI);
    const unsigned gb = (unsigned)std::min((size_t)need, (size_t)grid);
    k_mul_bn<TPI, L><<<gb, kBlock, 0, st>>>(kc, a, emag, el, out, count, scratch, wb, err, ctr);
  });
  return counted();
}

int resident_blocks_mul_bn(int S) {
  int r = 0;
  [&]() -> cudaError_t { HG_DISPATCH_S0(S, r = occupancy_blocks(k_mul_bn<TPI, L>)); return cudaSuccess; }();
  return r;
}

cudaError_t launch_sel_from_neg(const uint8_t* neg, int64_t* sel, size_t count, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  k_sel_from_neg<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(neg, sel, count);
  return counted();
}

cudaError_t launch_mul_const(int S, const KeyConst& kc, const uint32_t* in, const uint32_t* c, uint32_t* out,
                             size_t count, uint32_t* err, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  HG_DISPATCH_S0(S, k_mul_const<TPI, L><<<blocks_for(count, TPI), kBlock, 0, st>>>(kc, in, c, out, count, err));
  return counted();
}

cudaError_t launch_convert(int S, const KeyConst& kc, const uint32_t* in, uint32_t* out, size_t count,
                           int to_mont, uint32_t* err, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  HG_DISPATCH_S0(S,
                 k_convert<TPI, L><<<blocks_for(count, TPI), kBlock, 0, st>>>(kc, in, out, count, to_mont, err));
  return counted();
}

cudaError_t launch_reduce(int S, const KeyConst& kc, const uint32_t* in, size_t count, int chunk,
                          uint32_t* out, uint32_t* err, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  const size_t out_count = (count + chunk - 1) / chunk;
  HG_DISPATCH_S0(S,
                 k_reduce<TPI, L><<<blocks_for(out_count, TPI), kBlock, 0, st>>>(kc, in, count, chunk, out,
                                                                                 out_count, err));
  return counted();
}

cudaError_t launch_reduce_tree(int S, const KeyConst& kc, const uint32_t* in, size_t count, int chunk,
                               uint32_t* out, uint32_t* err, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  HG_DISPATCH_S0(S, {
    const size_t per_block = (size_t)(kBlock / TPI) * (size_t)chunk;
    const unsigned blocks = (unsigned)((count + per_block - 1) / per_block);
    k_reduce_tree<TPI, L><<<blocks, kBlock, 0, st>>>(kc, in, count, chunk, out, err);
  });
  return counted();
}

// The serving loop runs these kernels next to persistent batch kernels that
// take the largest shared-memory carveout; an SM changes its L1 / shared
// split only when it is idle, so a kernel preferring another split would wait
// for the long batches to drain.  All of them prefer the same split.
void server_prefer_shared_carveout() {
  auto set = [](const void* f) { cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, 100); };
#define HG_CARVE(TPI, L)                                                  \
  set((const void*)k_reduce_tree<TPI, L>);                                \
  set((const void*)k_reduce<TPI, L>);                                     \
  set((const void*)k_tree_leaves<TPI, L>);                                \
  set((const void*)k_tree_up<TPI, L>);                                    \
  set((const void*)k_tree_down<TPI, L>);                                  \
  set((const void*)k_tree_apply<TPI, L>);
  HG_CARVE(4, 16)
  HG_CARVE(8, 16)
  HG_CARVE(16, 12)
#undef HG_CARVE
}

size_t reduce_tree_outputs(int S, size_t count, int chunk) {
  const int tpi = S == 64 ? 4 : S == 128 ? 8 : 16;
  const size_t per_block = (size_t)(kBlock / tpi) * (size_t)chunk;
  return (count + per_block - 1) / per_block;
}

int reduce_tree_chunk(int S, size_t count, int sms) {
  const int tpi = S == 64 ? 4 : S == 128 ? 8 : 16;
  const size_t gpb = (size_t)(kBlock / tpi);
  // blocks of this instance resident on one SM (register-limited)
  int per_sm = 0;
  if (S == 64) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_reduce_tree<4, 16>, kBlock, 0);
  if (S == 128) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_reduce_tree<8, 16>, kBlock, 0);
  if (S == 192) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_reduce_tree<16, 12>, kBlock, 0);
  const size_t resident = (size_t)std::max(1, sms) * (size_t)std::max(1, per_sm) * gpb;
  // a few inputs per group: one block finishes the sum
  if (count <= 4 * gpb) return (int)((count + gpb - 1) / gpb);
  // more inputs than resident groups: one full wave, every group the same
  // number of inputs; fewer: one input per group (latency-bound levels)
  return (int)std::max<size_t>(1, (count + resident - 1) / resident);
}

cudaError_t launch_tree_leaves(int S, const KeyConst& kc, const uint32_t* in, const int64_t* sel, size_t count,
                               uint32_t* leaves, size_t padded, uint32_t* err, cudaStream_t st) {
  HG_DISPATCH_S0(S,
                 k_tree_leaves<TPI, L><<<blocks_for(padded, TPI), kBlock, 0, st>>>(kc, in, sel, count, leaves,
                                                                                   padded, err));
  return counted();
}

cudaError_t launch_tree_up(int S, const KeyConst& kc, const uint32_t* lower, uint32_t* upper, size_t upper_count,
                           cudaStream_t st) {
  HG_DISPATCH_S0(S,
                 k_tree_up<TPI, L><<<blocks_for(upper_count, TPI), kBlock, 0, st>>>(kc, lower, upper, upper_count));
  return counted();
}

cudaError_t launch_tree_down(int S, const KeyConst& kc, uint32_t* lower, const uint32_t* upper_inv,
                             size_t upper_count, cudaStream_t st) {
  HG_DISPATCH_S0(S,
                 k_tree_down<TPI, L><<<blocks_for(upper_count, TPI), kBlock, 0, st>>>(kc, lower, upper_inv,
                                                                                      upper_count));
  return counted();
}

cudaError_t launch_tree_apply(int S, const KeyConst& kc, const uint32_t* in, const int64_t* sel,
                              const uint32_t* leaves_inv, uint32_t* out, size_t count, cudaStream_t st) {
  HG_DISPATCH_S0(S,
                 k_tree_apply<TPI, L><<<blocks_for(count, TPI), kBlock, 0, st>>>(kc, in, sel, leaves_inv, out,
                                                                                 count));
  return counted();
}

cudaError_t launch_table_bases(int S, const KeyConst& kc, const uint32_t* hs_mont, uint32_t* bases,
                               cudaStream_t st) {
  HG_DISPATCH_S0(S, k_table_bases<TPI, L><<<1, 32, 0, st>>>(kc, hs_mont, bases));
  return counted();
}

cudaError_t launch_table_level(int S, const KeyConst& kc, uint32_t* table, const uint32_t* bases, int level,
                               cudaStream_t st) {
  size_t total;
  if (level < 0) {
    total = (size_t)kc.npos;
  } else {
    const size_t ent = (size_t)((1u << kc.w) - 1u);
    const size_t lo = (1ull << level) + 1ull;
    const size_t hi = std::min((size_t)(1ull << (level + 1)), ent);
    if (hi < lo) return cudaSuccess;
    total = (hi - lo + 1) * (size_t)kc.npos;
  }
  HG_DISPATCH_S0(S,
                 k_table_level<TPI, L><<<blocks_for(total, TPI), kBlock, 0, st>>>(kc, table, bases, level));
  return counted();
}

}  // namespace hg

// CRT decryption kernel (decryptor.cc:32-53): two groups of TP lanes per
// ciphertext, one per prime; persistent grid, each unit slot owning two
// odd-power tables in scratch and a hand-off buffer in shared memory; warps
// take ciphertexts from a launch-wide counter (next_work).
#include <algorithm>

#include "paillier_ops.cuh"

namespace hg {

namespace {
constexpr int kBlock = 128;

// Resident blocks per SM the compiler must fit (register budget).  The
// 2048-bit throughput layout (4 lanes x 16 limbs per side) is held at 96
// registers so five blocks fit instead of four: decryption 312 k/s -> 322
// k/s on 2^20 ciphertexts (the extra warps hide more of the dependent
// multiply-add latency; six blocks, 80 registers, spill and fall back to
// 315 k/s).  The 3072-bit layout (8 lanes x 12 limbs) likewise fits five
// blocks in 94 registers without spilling (a mixed-key stream dominated by
// 3072-bit decryptions: 428 k -> 433 k ops/s per call).  The other layouts
// keep the compiler's own budget.
constexpr int dec_min_blocks(int TP, int LP) { return ((TP == 4 && LP == 16) || (TP == 8 && LP == 12)) ? 5 : 1; }
}  // namespace

void count_launches(uint64_t n);

template <int TP, int LP>
__global__ void __launch_bounds__(kBlock, dec_min_blocks(TP, LP)) k_decrypt(KeyConst kc, SecConst sc, const uint32_t* __restrict__ ct,
                                                    size_t count, int64_t* __restrict__ out_i64,
                                                    uint8_t* __restrict__ out_ovf, uint32_t* __restrict__ out_mag,
                                                    uint8_t* __restrict__ out_neg, uint32_t* __restrict__ scratch,
                                                    uint32_t* err, unsigned long long* ctr, Codec cd) {
  constexpr int SP = TP * LP;
  constexpr int UPW = 32 / (2 * TP);  // ciphertexts per warp
  constexpr int UPB = kBlock / (2 * TP);
  __shared__ __align__(16) uint32_t ysm[UPB][2 * SP];
  const Group<TP> g;
  const int lane = threadIdx.x & 31;
  const int side = (lane / TP) & 1;
  const int unit_w = lane / (2 * TP);
  const int unit_b = threadIdx.x / (2 * TP);
  const int ntab = 1 << (sc.wd - 1);
  uint32_t* tb = scratch + (((size_t)blockIdx.x * UPB + unit_b) * 2 + side) * (size_t)ntab * SP + g.t * LP;
  for (size_t wbase = next_work(ctr, UPW); wbase < count; wbase = next_work(ctr, UPW)) {
    const size_t inst = wbase + unit_w;
    const bool active = inst < count;
    decrypt_one<TP, LP>(kc, sc, ct, active ? inst : count - 1, active, side, tb, ysm[unit_b], out_i64, out_ovf,
                        out_mag, out_neg, g, err, cd);
  }
}

template <typename K>
static int occupancy_blocks(K kernel) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kBlock, 0);
  return sms * (per > 0 ? per : 1);
}

int units_per_block_decrypt(int Sp, int variant) {
  const int tp = (Sp == 32) ? (variant ? 4 : 2) : (Sp == 64) ? (variant ? 8 : 4) : (variant ? 4 : 8);
  return kBlock / (2 * tp);
}

int resident_blocks_decrypt(int Sp, int variant) {
  int r = 0;
  [&]() -> cudaError_t {
    HG_DISPATCH_SPV(Sp, variant, r = occupancy_blocks(k_decrypt<TP, LP>));
    return cudaSuccess;
  }();
  return r;
}

// Batches up to one wave of the latency layout (a half warp per CRT side,
// one ciphertext per warp), and at most 12 per SM, run in that layout.
static size_t latency_wave_decrypt(int Sp) {
  static size_t cache[3] = {0, 0, 0};
  const int slot = Sp == 32 ? 0 : Sp == 64 ? 1 : 2;
  if (cache[slot] == 0) {
    size_t v = 0;
    [&]() -> cudaError_t {
      HG_DISPATCH_SPL(Sp, v = (size_t)occupancy_blocks(k_decrypt<TP, LP>) * (kBlock / 32));
      int dev = 0, sms = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      // at most 12 ciphertexts per SM (4096 took 18.3 ms in this layout
      // against 16.1 ms in the throughput layout on GB300, one 4.2 ms
      // against 10.2 ms)
      v = std::min(v, (size_t)12 * (size_t)sms);
      return cudaSuccess;
    }();
    cache[slot] = v;
  }
  return cache[slot];
}

cudaError_t launch_decrypt(int Sp, const KeyConst& kc, const SecConst& sc, const uint32_t* ct, size_t count,
                           int64_t* out_i64, uint8_t* out_ovf, uint32_t* out_mag, uint8_t* out_neg,
                           uint32_t* scratch, uint32_t* err, int grid, unsigned long long* ctr, cudaStream_t st,
                           const Codec& cd) {
  if (count == 0) return cudaSuccess;
  const cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(*ctr), st);
  if (e != cudaSuccess) return e;
  // the latency layout's unit slots must fit the scratch sized for `grid`
  // blocks of the throughput layout
  const size_t lat_blocks = (count + kBlock / 32 - 1) / (kBlock / 32);
  if (count <= latency_wave_decrypt(Sp) &&
      lat_blocks * (kBlock / 32) <= (size_t)grid * units_per_block_decrypt(Sp, sc.variant)) {
    HG_DISPATCH_SPL(Sp, k_decrypt<TP, LP><<<(unsigned)lat_blocks, kBlock, 0, st>>>(
                            kc, sc, ct, count, out_i64, out_ovf, out_mag, out_neg, scratch, err, ctr, cd));
    count_launches(1);
    return cudaGetLastError();
  }
  HG_DISPATCH_SPV(Sp, sc.variant, {
    const size_t upb = kBlock / (2 * TP);
    const unsigned need = (unsigned)((count + upb - 1) / upb);
    const unsigned gb = (unsigned)std::min((size_t)need, (size_t)grid);
    k_decrypt<TP, LP><<<gb, kBlock, 0, st>>>(kc, sc, ct, count, out_i64, out_ovf, out_mag, out_neg, scratch, err,
                                             ctr, cd);
  });
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace hg

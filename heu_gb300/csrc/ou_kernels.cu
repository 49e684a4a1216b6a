// Okamoto-Uchiyama decryption (heu/library/algorithms/ou/decryptor.cc:27-45):
//   m = L(c^t mod p^2) * gp_inv mod p,  L(u) = (u - 1) / p,  centred at p/2.
// One group of TP lanes per ciphertext, persistent grid; the exponent t (a
// prime factor of p - 1) is one shared sliding-window program.  Encryption
// and every evaluator operation run on the generic Montgomery kernels over n
// (fixed-base tables for G, G^-1 and H), so this file holds only the part
// that differs from ZPaillier.
#include <algorithm>

#include "paillier_ops.cuh"

namespace hg {

namespace {
constexpr int kBlock = 128;
}

void count_launches(uint64_t n);

// (u - 1) / p * gp_inv mod p, centred: one lane, H-limb serial arithmetic
template <int H>
__device__ __noinline__ void ou_tail(const OuConst& oc, const uint32_t* u, size_t i, bool active,
                                     int64_t* __restrict__ out_i64, uint8_t* __restrict__ out_ovf,
                                     uint32_t* __restrict__ out_mag, uint8_t* __restrict__ out_neg) {
  uint32_t t1[H], Lv[H], m[H];
  uint64_t br = 1;
#pragma unroll 1
  for (int j = 0; j < H; ++j) {
    const uint64_t v = (uint64_t)u[j] - br;
    t1[j] = (uint32_t)v;
    br = (v >> 63) & 1ull;
  }
  // exact division by p: low H limbs of (u - 1) times p^-1 mod 2^(32H)
#pragma unroll 1
  for (int j = 0; j < H; ++j) Lv[j] = 0;
#pragma unroll 1
  for (int a = 0; a < H; ++a) {
    uint64_t c = 0;
    const uint32_t ta = t1[a];
#pragma unroll 1
    for (int b = 0; a + b < H; ++b) {
      c += (uint64_t)ta * oc.pinv[b] + Lv[a + b];
      Lv[a + b] = (uint32_t)c;
      c >>= 32;
    }
  }
  s_montmul<H>(m, Lv, oc.gpR, oc.P, oc.np1);
  // m > p/2 => m - p (decryptor.cc:40-43)
  bool gt = false;
#pragma unroll 1
  for (int j = H - 1; j >= 0; --j) {
    if (m[j] != oc.phalf[j]) {
      gt = m[j] > oc.phalf[j];
      break;
    }
  }
  if (gt) {
    int64_t b2 = 0;
#pragma unroll 1
    for (int j = 0; j < H; ++j) {
      const int64_t v = (int64_t)oc.P[j] - m[j] - b2;
      b2 = v < 0;
      m[j] = (uint32_t)v;
    }
  }
  if (!active) return;
  if (out_mag) {
#pragma unroll 1
    for (int j = 0; j < H; ++j) out_mag[i * H + j] = m[j];
    out_neg[i] = gt ? 1 : 0;
  }
  if (out_i64) {
    bool fits = true;
#pragma unroll 1
    for (int j = 2; j < H; ++j) fits &= (m[j] == 0u);
    const uint64_t mag = (uint64_t)m[0] | ((uint64_t)m[1] << 32);
    if (gt) {
      fits &= mag <= (1ull << 63);
      out_i64[i] = (int64_t)((uint64_t)0 - mag);
    } else {
      fits &= mag < (1ull << 63);
      out_i64[i] = (int64_t)mag;
    }
    if (out_ovf) out_ovf[i] = fits ? 0 : 1;
  }
}

// S: limbs of a ciphertext (mod n); SP = TP * LP: limbs of the p^2 arithmetic
template <int TP, int LP, int S>
__global__ void __launch_bounds__(kBlock) k_ou_decrypt(KeyConst kc, OuConst oc, const uint32_t* __restrict__ ct,
                                                       size_t count, int64_t* __restrict__ out_i64,
                                                       uint8_t* __restrict__ out_ovf, uint32_t* __restrict__ out_mag,
                                                       uint8_t* __restrict__ out_neg, uint32_t* __restrict__ scratch,
                                                       uint32_t* err, unsigned long long* ctr) {
  constexpr int SP = TP * LP;
  static_assert(S <= 2 * SP, "ciphertext must fit the wide reduction");
  constexpr int UPW = 32 / TP;
  constexpr int UPB = kBlock / TP;
  __shared__ __align__(16) uint32_t ysm[UPB][SP];
  const Group<TP> g;
  const int lane = threadIdx.x & 31;
  const int unit_w = lane / TP;
  const int unit_b = threadIdx.x / TP;
  const int ntab = 1 << (oc.wd - 1);
  uint32_t* tb = scratch + ((size_t)blockIdx.x * UPB + unit_b) * (size_t)ntab * SP + g.t * LP;
  uint32_t N[LP];
  load_slice<LP>(N, oc.P2 + g.t * LP);
  for (size_t wbase = next_work(ctr, UPW); wbase < count; wbase = next_work(ctr, UPW)) {
    const size_t inst = wbase + unit_w;
    const bool active = inst < count;
    const size_t i = active ? inst : count - 1;
    // the ciphertext as a 2*SP-limb value (limbs at and above S are zero)
    uint32_t lo[LP], hi[LP];
#pragma unroll
    for (int j = 0; j < LP; ++j) {
      const int a = g.t * LP + j, b = SP + g.t * LP + j;
      lo[j] = a < S ? ct[i * S + a] : 0u;
      hi[j] = b < S ? ct[i * S + b] : 0u;
    }
    {
      // validate 0 <= c < n (decryptor.cc:16-18)
      uint32_t Nlo[LP], Nhi[LP], d[LP], e2[LP];
#pragma unroll
      for (int j = 0; j < LP; ++j) {
        const int a = g.t * LP + j, b = SP + g.t * LP + j;
        Nlo[j] = a < S ? kc.N[a] : 0u;
        Nhi[j] = b < S ? kc.N[b] : 0u;
      }
      const uint32_t b_lo = sub_full<TP, LP>(d, lo, Nlo, g);
      (void)sub_full<TP, LP>(e2, hi, Nhi, g);
      const bool hi_lt = less_than<TP, LP>(hi, Nhi, g);
      const bool hi_eq = is_zero<TP, LP>(e2, g);
      const bool ok = hi_lt || (hi_eq && b_lo);
      if (active && !ok && g.t == 0) atomicOr(err, kErrCtRange);
    }
    // c*R_n mod p^2 -> c*R_p mod p^2: REDC, then one product with R_p^3 / R_n
    uint32_t x[LP], K[LP];
    mont_redc_wide<TP, LP>(x, lo, hi, N, oc.np2, g);
    load_slice<LP>(K, oc.Kfix + g.t * LP);
    mont_mul<TP, LP>(x, x, K, N, oc.np2, g);
    store_slice<LP>(tb, x);
    uint32_t x2[LP], cur[LP];
    mont_mul<TP, LP>(x2, x, x, N, oc.np2, g);
    copy_slice<LP>(cur, x);
#pragma unroll 1
    for (int t = 1; t < ntab; ++t) {
      mont_mul<TP, LP>(cur, cur, x2, N, oc.np2, g);
      store_slice<LP>(tb + (size_t)t * SP, cur);
    }
    uint32_t acc[LP];
    load_slice<LP>(acc, tb + (size_t)oc.start * SP);
#pragma unroll 1
    for (int s = 0; s < oc.prog_len; ++s) {
      const uint16_t op = oc.prog[s];
      uint32_t B[LP];
      if (op < kOpNop) {
        load_slice<LP>(B, tb + (size_t)op * SP);
      } else {
        copy_slice<LP>(B, acc);
      }
      uint32_t res[LP];
      mont_mul<TP, LP>(res, acc, B, N, oc.np2, g);
      if (op != kOpNop) copy_slice<LP>(acc, res);
    }
    mont_redc<TP, LP>(acc, acc, N, oc.np2, g);
#pragma unroll
    for (int j = 0; j < LP; ++j) ysm[unit_b][g.t * LP + j] = acc[j];
    __syncwarp();
    if (g.t == 0) ou_tail<SP / 2>(oc, ysm[unit_b], i, active, out_i64, out_ovf, out_mag, out_neg);
    __syncwarp();
  }
}

// G^m for signed m = G^(m+) * (G^-1)^(m-): split each plaintext into the two
// non-negative exponents (encryptor.cc:99-104 picks the table by sign).
// From int64 values (negated when `negate`), as 2-limb exponents.
__global__ void k_ou_split_i64(const int64_t* __restrict__ p, int negate, uint32_t* __restrict__ ep,
                               uint32_t* __restrict__ en, size_t count) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int64_t v = p[i];
  const bool neg = negate ? (v > 0) : (v < 0);
  const uint64_t mag = v < 0 ? (uint64_t)0 - (uint64_t)v : (uint64_t)v;
  const uint64_t a = neg ? 0ull : mag, b = neg ? mag : 0ull;
  ep[2 * i] = (uint32_t)a;
  ep[2 * i + 1] = (uint32_t)(a >> 32);
  en[2 * i] = (uint32_t)b;
  en[2 * i + 1] = (uint32_t)(b >> 32);
}

// From magnitudes of `limbs` limbs with sign flags; |m| > maxpt raises the
// plaintext range error (encryptor.cc:95-97).
__global__ void k_ou_split_mag(const uint32_t* __restrict__ mag, const uint8_t* __restrict__ neg, int limbs,
                               const uint32_t* __restrict__ maxpt, uint32_t* __restrict__ ep,
                               uint32_t* __restrict__ en, size_t count, uint32_t* err) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const uint32_t* x = mag + i * limbs;
  int cmp = 0;
  for (int j = limbs - 1; j >= 0 && cmp == 0; --j) cmp = (x[j] > maxpt[j]) - (x[j] < maxpt[j]);
  if (cmp > 0) atomicOr(err, kErrPtRange);
  const bool ng = neg[i] != 0;
  for (int j = 0; j < limbs; ++j) {
    ep[i * limbs + j] = ng ? 0u : x[j];
    en[i * limbs + j] = ng ? x[j] : 0u;
  }
}

cudaError_t launch_ou_split_i64(const int64_t* p, int negate, uint32_t* ep, uint32_t* en, size_t count,
                                cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  k_ou_split_i64<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(p, negate, ep, en, count);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_ou_split_mag(const uint32_t* mag, const uint8_t* neg, int limbs, const uint32_t* maxpt,
                                uint32_t* ep, uint32_t* en, size_t count, uint32_t* err, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  k_ou_split_mag<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(mag, neg, limbs, maxpt, ep, en, count, err);
  count_launches(1);
  return cudaGetLastError();
}

template <typename K>
static int occupancy_blocks(K kernel) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kBlock, 0);
  return sms * (per > 0 ? per : 1);
}

// (ciphertext limbs, p^2 limbs) -> (TP, LP); the three OU key sizes
#define HG_DISPATCH_OU(S, SP, ...)                                                   \
  if ((S) == 64 && (SP) == 32) {                                                     \
    constexpr int TP = 2, LP = 16, SC = 64;                                          \
    __VA_ARGS__;                                                                     \
  } else if ((S) == 128 && (SP) == 64) {                                             \
    constexpr int TP = 4, LP = 16, SC = 128;                                         \
    __VA_ARGS__;                                                                     \
  } else if ((S) == 128 && (SP) == 96) {                                             \
    constexpr int TP = 8, LP = 12, SC = 128;                                         \
    __VA_ARGS__;                                                                     \
  } else {                                                                           \
    return cudaErrorInvalidValue;                                                    \
  }

cudaError_t ou_decrypt_geometry(int S, int Sp, int* grid, int* units_per_block) {
  HG_DISPATCH_OU(S, Sp, {
    *grid = occupancy_blocks(k_ou_decrypt<TP, LP, SC>);
    *units_per_block = kBlock / TP;
  });
  return cudaSuccess;
}

cudaError_t launch_ou_decrypt(int S, const KeyConst& kc, const OuConst& oc, const uint32_t* ct, size_t count,
                              int64_t* out_i64, uint8_t* out_ovf, uint32_t* out_mag, uint8_t* out_neg,
                              uint32_t* scratch, uint32_t* err, int grid, unsigned long long* ctr,
                              cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  const cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(*ctr), st);
  if (e != cudaSuccess) return e;
  HG_DISPATCH_OU(S, oc.Sp, {
    const size_t upb = kBlock / TP;
    const unsigned need = (unsigned)((count + upb - 1) / upb);
    const unsigned gb = (unsigned)std::min((size_t)need, (size_t)grid);
    k_ou_decrypt<TP, LP, SC><<<gb, kBlock, 0, st>>>(kc, oc, ct, count, out_i64, out_ovf, out_mag, out_neg, scratch,
                                                   err, ctr);
  });
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace hg

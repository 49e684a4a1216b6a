// Distributed Montgomery squaring for the lane layout of mont.cuh.
//
// A square needs only half of the cross products a_i a_j (i < j, doubled)
// plus the diagonal terms.  In the CIOS loop of mont_mul every lane of the
// group multiplies its slice by every limb, so the symmetry cannot be used
// there without idle lanes.  Here the product a^2 (2S limbs) is formed first
// from per-lane block products of equal shape, then reduced with the
// separated Montgomery reduction (mont_redc_wide):
//   round 0:        lane t squares its own slice A_t (cross products once,
//                   doubled, plus squares): L(L+1)/2 multiplications;
//   round r < P/2:  lane t multiplies A_t by A_(t+r mod P) and doubles it
//                   (the mirror block is never formed): L^2;
//   round P/2:      lane t multiplies A_t by A_(t+P/2 mod P) once (each such
//                   block is formed by both of its lanes, once each): L^2.
// Per lane that is L(L+1)/2 + (P/2) L^2 multiplications instead of the
// P L^2 of the CIOS product rows.  Each block lands at slice t + u (and the
// next) of a^2; it is staged in shared memory and every lane adds the (at
// most two) pieces that fall into the two slices it owns (slice t of the low
// half, slice t of the high half), keeping a lazy carry word per slice.  The
// carries are settled with a ballot lookahead over the 2P slices.
#pragma once
#include "mont.cuh"

namespace hg {

// q[0..2L) = a * b (one lane, schoolbook rows)
template <int L>
__device__ __forceinline__ void block_mul(uint32_t (&q)[2 * L + 1], const uint32_t (&a)[L], const uint32_t (&b)[L]) {
#pragma unroll
  for (int k = 0; k < 2 * L + 1; ++k) q[k] = 0u;
#pragma unroll
  for (int i = 0; i < L; ++i) {
    uint64_t c = 0;
#pragma unroll
    for (int j = 0; j < L; ++j) {
      const uint64_t t = (uint64_t)a[i] * b[j] + q[i + j] + c;
      q[i + j] = (uint32_t)t;
      c = t >> 32;
    }
    q[i + L] = (uint32_t)c;
  }
}

// stage[k][lane] = limb k of a * b (doubled when dbl), k = 0..2L, written as
// soon as each limb is final (after row k of the schoolbook product), so only
// a window of L + 1 limbs lives in registers.
template <int L>
__device__ __forceinline__ void block_mul_stage(uint32_t* stage, int lane, const uint32_t (&a)[L],
                                                const uint32_t (&b)[L], bool dbl) {
  uint32_t w[L + 1];
#pragma unroll
  for (int k = 0; k <= L; ++k) w[k] = 0u;
  uint32_t prev = 0u;
  auto put = [&](int k, uint32_t v) {
    stage[(size_t)k * 32 + lane] = dbl ? __funnelshift_l(prev, v, 1) : v;
    prev = v;
  };
#pragma unroll
  for (int i = 0; i < L; ++i) {
    uint64_t c = 0;
#pragma unroll
    for (int j = 0; j < L; ++j) {
      const uint64_t t = (uint64_t)a[i] * b[j] + w[j] + c;
      w[j] = (uint32_t)t;
      c = t >> 32;
    }
    w[L] = (uint32_t)c;
    put(i, w[0]);
#pragma unroll
    for (int k = 0; k < L; ++k) w[k] = w[k + 1];
    w[L] = 0u;
  }
#pragma unroll
  for (int k = 0; k < L; ++k) put(L + k, w[k]);
  stage[(size_t)(2 * L) * 32 + lane] = dbl ? (prev >> 31) : 0u;
}

// q[0..2L) = a^2 (one lane): cross products once, doubled, plus squares
template <int L>
__device__ __forceinline__ void block_sqr(uint32_t (&q)[2 * L + 1], const uint32_t (&a)[L]) {
#pragma unroll
  for (int k = 0; k < 2 * L + 1; ++k) q[k] = 0u;
#pragma unroll
  for (int i = 0; i < L - 1; ++i) {
    uint64_t c = 0;
#pragma unroll
    for (int j = i + 1; j < L; ++j) {
      const uint64_t t = (uint64_t)a[i] * a[j] + q[i + j] + c;
      q[i + j] = (uint32_t)t;
      c = t >> 32;
    }
    q[i + L] = (uint32_t)c;
  }
  // double the cross products (below a^2 / 2, so no bit leaves 2L limbs)
#pragma unroll
  for (int k = 2 * L - 1; k > 0; --k) q[k] = __funnelshift_l(q[k - 1], q[k], 1);
  q[0] <<= 1;
  uint64_t c = 0;
#pragma unroll
  for (int i = 0; i < L; ++i) {
    const uint64_t t = (uint64_t)a[i] * a[i] + q[2 * i] + c;
    q[2 * i] = (uint32_t)t;
    const uint64_t u = (t >> 32) + q[2 * i + 1];
    q[2 * i + 1] = (uint32_t)u;
    c = u >> 32;
  }
}

// slice of a^2 at which lane s's block of round rd starts
template <int P>
__device__ __forceinline__ int sqr_block_slice(int s, int rd) {
  return rd == 0 ? 2 * s : s + ((s + rd) & (P - 1));
}

// The slice x (lazy carry cw) accumulated in shared memory at acc (column
// `lane`, rows 0..L-1) += the pieces of round rd that fall into x: the low
// half of a block starting at x, or the high half (plus its carry limb,
// which sits where x's own carry goes) of a block starting at x - 1.
template <int P, int L>
__device__ __forceinline__ void sqr_gather(uint32_t* acc, uint32_t& cw, int x, int rd, const uint32_t* stage,
                                           int base, int lane) {
  int src0 = -1, half0 = 0, src1 = -1, half1 = 0;
#pragma unroll
  for (int s = 0; s < P; ++s) {
    const int sg = sqr_block_slice<P>(s, rd);
    const int h = (sg == x) ? 0 : (sg + 1 == x) ? 1 : -1;
    if (h >= 0) {
      if (src0 < 0) {
        src0 = s;
        half0 = h;
      } else {
        src1 = s;
        half1 = h;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int src = k == 0 ? src0 : src1;
    const int half = k == 0 ? half0 : half1;
    const bool use = src >= 0;
    const uint32_t* p = stage + (size_t)(half * L) * 32 + base + (use ? src : 0);
    uint32_t v = use ? p[0] : 0u;
    acc[lane] = add_cc(acc[lane], v);
#pragma unroll
    for (int j = 1; j < L; ++j) {
      v = use ? p[(size_t)j * 32] : 0u;
      acc[(size_t)j * 32 + lane] = addc_cc(acc[(size_t)j * 32 + lane], v);
    }
    const uint32_t cout = addc(0u, 0u);
    const uint32_t top = (use && half == 1) ? stage[(size_t)(2 * L) * 32 + base + src] : 0u;
    cw += cout + top;
  }
}

// r = a^2 * R^-1 mod N for a < N.  smem: this warp's shared scratch of
// sqr_smem_words(L) words (block staging and the 2S-limb accumulator).
// r may alias a.
template <int L>
__host__ __device__ constexpr int sqr_smem_words() {
  return (4 * L + 1) * 32;
}

template <int TPI, int L>
__device__ __forceinline__ void mont_sqr(uint32_t (&r)[L], const uint32_t (&a)[L], const uint32_t (&n)[L],
                                         uint32_t np, const Group<TPI>& g, uint32_t* smem) {
  constexpr int P = TPI;
  const int lane = threadIdx.x & 31;
  uint32_t* stage = smem;                        // (2L + 1) x 32
  uint32_t* acc = smem + (size_t)(2 * L + 1) * 32;  // 2L x 32: low slice rows 0..L-1, high slice rows L..2L-1
#pragma unroll
  for (int j = 0; j < 2 * L; ++j) acc[(size_t)j * 32 + lane] = 0u;
  uint32_t clo = 0u, chi = 0u;
  {
    uint32_t q[2 * L + 1];
    block_sqr<L>(q, a);
#pragma unroll
    for (int k = 0; k < 2 * L + 1; ++k) stage[(size_t)k * 32 + lane] = q[k];
  }
  __syncwarp();
  sqr_gather<P, L>(acc, clo, (int)g.t, 0, stage, (int)g.base, lane);
  sqr_gather<P, L>(acc + (size_t)L * 32, chi, (int)g.t + P, 0, stage, (int)g.base, lane);
#pragma unroll 1
  for (int rd = 1; rd <= P / 2; ++rd) {
    uint32_t b[L];
    const int src = (int)g.base + (((int)g.t + rd) & (P - 1));
#pragma unroll
    for (int j = 0; j < L; ++j) b[j] = __shfl_sync(kFull, a[j], src);
    __syncwarp();  // the previous round's gathers have read the stage
    // below P/2 the mirror block is not formed: this one counts twice
    block_mul_stage<L>(stage, lane, a, b, rd < P / 2);
    __syncwarp();
    sqr_gather<P, L>(acc, clo, (int)g.t, rd, stage, (int)g.base, lane);
    sqr_gather<P, L>(acc + (size_t)L * 32, chi, (int)g.t + P, rd, stage, (int)g.base, lane);
  }
  uint32_t lo[L], hi[L];
#pragma unroll
  for (int j = 0; j < L; ++j) {
    lo[j] = acc[(size_t)j * 32 + lane];
    hi[j] = acc[(size_t)(L + j) * 32 + lane];
  }
  __syncwarp();
  // settle: the carry word of slice x belongs to slice x + 1 (low slices
  // 0..P-1 then high slices 0..P-1; the top one is zero since a^2 < 2^(64 S))
  uint32_t in_lo = __shfl_up_sync(kFull, clo, 1, TPI);
  uint32_t in_hi = __shfl_up_sync(kFull, chi, 1, TPI);
  const uint32_t last_lo = __shfl_sync(kFull, clo, P - 1, TPI);
  if (g.t == 0) {
    in_lo = 0u;
    in_hi = last_lo;
  }
  lo[0] = add_cc(lo[0], in_lo);
#pragma unroll
  for (int j = 1; j < L; ++j) lo[j] = addc_cc(lo[j], 0u);
  const uint32_t glo = addc(0u, 0u);
  hi[0] = add_cc(hi[0], in_hi);
#pragma unroll
  for (int j = 1; j < L; ++j) hi[j] = addc_cc(hi[j], 0u);
  const uint32_t ghi = addc(0u, 0u);
  uint32_t all_lo = lo[0], all_hi = hi[0];
#pragma unroll
  for (int j = 1; j < L; ++j) {
    all_lo &= lo[j];
    all_hi &= hi[j];
  }
  // lookahead over 2P slices: bit i < P = low slice i, bit P + i = high slice i
  const uint32_t Gl = __ballot_sync(kFull, glo != 0u), Pl = __ballot_sync(kFull, all_lo == kFull);
  const uint32_t Gh = __ballot_sync(kFull, ghi != 0u), Ph = __ballot_sync(kFull, all_hi == kFull);
  const uint64_t msk = (P == 32) ? 0xffffffffull : ((1ull << P) - 1ull);
  const uint64_t G = ((uint64_t)(Gl >> g.base) & msk) | (((uint64_t)(Gh >> g.base) & msk) << P);
  const uint64_t Pp = ((uint64_t)(Pl >> g.base) & msk) | (((uint64_t)(Ph >> g.base) & msk) << P);
  const uint64_t c = ((G | Pp) + G) ^ Pp;
  const uint32_t ci_lo = (uint32_t)(c >> g.t) & 1u;
  const uint32_t ci_hi = (uint32_t)(c >> (g.t + P)) & 1u;
  lo[0] = add_cc(lo[0], ci_lo);
#pragma unroll
  for (int j = 1; j < L; ++j) lo[j] = addc_cc(lo[j], 0u);
  (void)addc(0u, 0u);
  hi[0] = add_cc(hi[0], ci_hi);
#pragma unroll
  for (int j = 1; j < L; ++j) hi[j] = addc_cc(hi[j], 0u);
  (void)addc(0u, 0u);
  mont_redc_wide<TPI, L>(r, lo, hi, n, np, g);
}

}  // namespace hg

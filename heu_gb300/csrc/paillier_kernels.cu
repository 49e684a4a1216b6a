// Paillier (DJN variant, HEU paillier_z semantics) kernels for sm_103a.
//
// Every ciphertext is handled by a group of TPI lanes (mont.cuh).  The
// kernels keep warps converged: loop trip counts are uniform per warp, tails
// compute on a clamped index and skip their stores, and per-instance choices
// (square vs multiply, which table entry) only change the data a uniform
// Montgomery multiplication consumes.
#include <algorithm>
#include <atomic>

#include "mont.cuh"
#include "paillier_kernels.cuh"

namespace hg {

constexpr int kBlock = 128;  // threads per block for every kernel here

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t abs_i64(int64_t v) {
  return v < 0 ? (uint64_t)0 - (uint64_t)v : (uint64_t)v;
}

// Extract `w` bits of a little-endian limb array starting at bit `off`.
__device__ __forceinline__ uint32_t get_bits(const uint32_t* __restrict__ x, int nlimbs, int off, int w) {
  const int li = off >> 5, sh = off & 31;
  uint64_t v = (li < nlimbs) ? x[li] : 0u;
  if (li + 1 < nlimbs) v |= (uint64_t)x[li + 1] << 32;
  return (uint32_t)(v >> sh) & ((w >= 32) ? 0xffffffffu : ((1u << w) - 1u));
}

// gm = Montgomery form of (1 + m*n) mod N for m = (neg ? -A : A), A < n:
//   X = MM(A, n*R^2) = A*n*R;  gm = R + X (m >= 0) or R + (N - X) (m < 0).
template <int TPI, int L>
__device__ __forceinline__ void to_gm(uint32_t (&gm)[L], const uint32_t (&A)[L], bool neg,
                                      const uint32_t (&N)[L], const KeyConst& kc, const Group<TPI>& g) {
  uint32_t B[L], X[L];
  load_slice<L>(B, kc.nR2 + g.t * L);
  mont_mul<TPI, L>(X, A, B, N, kc.np, g);
  uint32_t negX[L];
  (void)sub_full<TPI, L>(negX, N, X, g);
  select_slice<L>(X, neg, negX, X);
  load_slice<L>(B, kc.R1 + g.t * L);
  mod_add<TPI, L>(gm, B, X, N, g);
}

template <int TPI, int L>
__device__ __forceinline__ void check_ct(const uint32_t (&x)[L], const uint32_t (&N)[L], bool active,
                                         const Group<TPI>& g, uint32_t* err) {
  const bool ok = less_than<TPI, L>(x, N, g);
  if (active && !ok && g.t == 0) atomicOr(err, kErrCtRange);
}

// ---------------------------------------------------------------------------
// Encrypt / EncryptZero / Randomize:
//   acc = gm(m) | R | ct_in;  acc *= prod_pos table[pos][digit_pos(r)]
// (encryptor.cc:26-56, evaluator.cc:25-28)
// ---------------------------------------------------------------------------
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_encrypt(KeyConst kc, EncMode mode, const int64_t* __restrict__ m,
                                                    const uint32_t* __restrict__ m_mag,
                                                    const uint8_t* __restrict__ m_neg,
                                                    const uint32_t* __restrict__ r,
                                                    const uint32_t* __restrict__ ct_in, uint32_t* __restrict__ out,
                                                    size_t count, uint32_t* err) {
  constexpr int S = TPI * L;
  constexpr int IPB = kBlock / TPI;
  const Group<TPI> g;
  const int warp_first = (threadIdx.x >> 5) * (32 / TPI);
  const size_t stride = (size_t)gridDim.x * IPB;
  uint32_t N[L];
  load_slice<L>(N, kc.N + g.t * L);
  const size_t ent = (size_t)((1u << kc.w) - 1u);
  for (size_t wbase = (size_t)blockIdx.x * IPB + warp_first; wbase < count; wbase += stride) {
    const size_t inst = wbase + (threadIdx.x & 31) / TPI;
    const bool active = inst < count;
    const size_t i = active ? inst : count - 1;
    uint32_t acc[L];
    if (mode == EncMode::kEncrypt) {
      uint32_t A[L];
      bool neg;
      if (m_mag != nullptr) {
        // |m| has S/2 limbs; lanes above them hold zeros
        uint32_t NH[L], d[L];
        if (g.t * L < S / 2) {
          load_slice<L>(A, m_mag + i * (S / 2) + g.t * L);
          load_slice<L>(NH, kc.nhalf + g.t * L);
        } else {
#pragma unroll
          for (int j = 0; j < L; ++j) A[j] = NH[j] = 0u;
        }
        neg = m_neg[i] != 0;
        // encryptor.cc:38-40: |m| <= n/2
        const bool too_big = sub_full<TPI, L>(d, NH, A, g) != 0u;
        if (active && too_big && g.t == 0) atomicOr(err, kErrPtRange);
      } else {
        set_u64<TPI, L>(A, g, abs_i64(m[i]));
        neg = m[i] < 0;
      }
      to_gm<TPI, L>(acc, A, neg, N, kc, g);
    } else if (mode == EncMode::kZero) {
      load_slice<L>(acc, kc.R1 + g.t * L);
    } else {
      load_slice<L>(acc, ct_in + i * S + g.t * L);
      check_ct<TPI, L>(acc, N, active, g, err);
    }
    const uint32_t* ri = r + i * kc.rlimbs;
#pragma unroll 1
    for (int pos = 0; pos < kc.npos; ++pos) {
      const int off = pos * kc.w;
      const int w = min(kc.w, kc.rbits - off);
      const uint32_t dg = get_bits(ri, kc.rlimbs, off, w);
      uint32_t B[L];
      const uint32_t* src = dg ? kc.table + ((size_t)pos * ent + (dg - 1u)) * S : kc.R1;
      load_slice<L>(B, src + g.t * L);
      mont_mul<TPI, L>(acc, acc, B, N, kc.np, g);
    }
    if (active) store_slice<L>(out + i * S + g.t * L, acc);
  }
}

// ---------------------------------------------------------------------------
// Add(ct, ct): MulMod of Montgomery residues (evaluator.cc:30-44)
// ---------------------------------------------------------------------------
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_add(KeyConst kc, const uint32_t* __restrict__ a,
                                                const uint32_t* __restrict__ b, uint32_t* __restrict__ out,
                                                size_t count, uint32_t* err) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  if (wfirst >= count) return;  // whole warp idle
  const bool active = inst < count;
  const size_t i = active ? inst : count - 1;
  uint32_t N[L], A[L], B[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(A, a + i * S + g.t * L);
  load_slice<L>(B, b + i * S + g.t * L);
  check_ct<TPI, L>(A, N, active, g, err);
  check_ct<TPI, L>(B, N, active, g, err);
  mont_mul<TPI, L>(A, A, B, N, kc.np, g);
  if (active) store_slice<L>(out + i * S + g.t * L, A);
}

// ---------------------------------------------------------------------------
// Add(ct, pt) / Sub(ct, pt): a * (1 + n*p) (evaluator.cc:46-76)
// ---------------------------------------------------------------------------
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_add_plain(KeyConst kc, const uint32_t* __restrict__ a,
                                                      const int64_t* __restrict__ p, int neg_p,
                                                      uint32_t* __restrict__ out, size_t count, uint32_t* err) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  if (wfirst >= count) return;
  const bool active = inst < count;
  const size_t i = active ? inst : count - 1;
  uint32_t N[L], A[L], G[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(A, a + i * S + g.t * L);
  check_ct<TPI, L>(A, N, active, g, err);
  const int64_t pv = p[i];
  // Sub(ct, pt) adds -p (evaluator.cc:74-76); the magnitude covers INT64_MIN
  uint32_t Am[L];
  set_u64<TPI, L>(Am, g, abs_i64(pv));
  to_gm<TPI, L>(G, Am, (pv < 0) != (neg_p != 0), N, kc, g);
  mont_mul<TPI, L>(A, A, G, N, kc.np, g);
  if (active) store_slice<L>(out + i * S + g.t * L, A);
}

// ---------------------------------------------------------------------------
// Mul(ct, k) for 64-bit k: c^|k| by left-to-right sliding windows (odd
// powers c, c^3, .., c^(2^wm - 1) kept in scratch).  k = 0 gives the
// Montgomery identity (evaluator.cc:105-106).  k < 0 is finished by the
// batch inverse on the host side of the launch (evaluator.cc:119-121).
// ---------------------------------------------------------------------------
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_mul(KeyConst kc, const uint32_t* __restrict__ a,
                                                const int64_t* __restrict__ kk, uint32_t* __restrict__ out,
                                                size_t count, uint32_t* __restrict__ scratch, int wm,
                                                uint32_t* err) {
  constexpr int S = TPI * L;
  constexpr int IPB = kBlock / TPI;
  const Group<TPI> g;
  const int lane_inst = (threadIdx.x & 31) / TPI;
  const int warp_first = (threadIdx.x >> 5) * (32 / TPI);
  const size_t stride = (size_t)gridDim.x * IPB;
  const int ntab = 1 << (wm - 1);
  uint32_t* tb = scratch + ((size_t)blockIdx.x * IPB + warp_first + lane_inst) * (size_t)ntab * S + g.t * L;
  uint32_t N[L];
  load_slice<L>(N, kc.N + g.t * L);
  for (size_t wbase = (size_t)blockIdx.x * IPB + warp_first; wbase < count; wbase += stride) {
    const size_t inst = wbase + lane_inst;
    const bool active = inst < count;
    const size_t i = active ? inst : count - 1;
    const uint64_t e = abs_i64(kk[i]);
    uint32_t x[L];
    load_slice<L>(x, a + i * S + g.t * L);
    check_ct<TPI, L>(x, N, active, g, err);
    // odd powers
    store_slice<L>(tb, x);
    uint32_t x2[L], cur[L];
    mont_mul<TPI, L>(x2, x, x, N, kc.np, g);
    copy_slice<L>(cur, x);
#pragma unroll 1
    for (int t = 1; t < ntab; ++t) {
      mont_mul<TPI, L>(cur, cur, x2, N, kc.np, g);
      store_slice<L>(tb + (size_t)t * S, cur);
    }
    // first window
    int pos = (e == 0) ? -1 : 63 - __clzll((long long)e);
    uint32_t acc[L];
    int sq = 0, mulidx = -1;
    if (pos >= 0) {
      int j = max(pos - wm + 1, 0);
      while (!((e >> j) & 1ull)) ++j;
      const uint32_t val = (uint32_t)((e >> j) & ((1ull << (pos - j + 1)) - 1ull));
      load_slice<L>(acc, tb + (size_t)((val - 1) >> 1) * S);
      pos = j - 1;
    } else {
      load_slice<L>(acc, kc.R1 + g.t * L);
    }
    // remaining bits: one Montgomery multiplication per step for every group
#pragma unroll 1
    while (true) {
      int op = 0;  // 0 = none, 1 = square, 2 = multiply by table[mulidx]
      if (sq > 0) {
        op = 1;
        --sq;
      } else if (mulidx >= 0) {
        op = 2;
      } else if (pos >= 0) {
        if (!((e >> pos) & 1ull)) {
          op = 1;
          --pos;
        } else {
          int j = max(pos - wm + 1, 0);
          while (!((e >> j) & 1ull)) ++j;
          const uint32_t val = (uint32_t)((e >> j) & ((1ull << (pos - j + 1)) - 1ull));
          sq = pos - j;  // squarings still owed after this one
          mulidx = (int)((val - 1) >> 1);
          op = 1;
          pos = j - 1;
        }
      }
      if (!__any_sync(kFull, op != 0)) break;
      uint32_t B[L];
      if (op == 2) {
        load_slice<L>(B, tb + (size_t)mulidx * S);
        mulidx = -1;
      } else {
        copy_slice<L>(B, acc);
      }
      uint32_t res[L];
      mont_mul<TPI, L>(res, acc, B, N, kc.np, g);
      if (op != 0) copy_slice<L>(acc, res);
    }
    if (active) store_slice<L>(out + i * S + g.t * L, acc);
  }
}

// ---------------------------------------------------------------------------
// Decrypt (decryptor.cc:32-53): two groups per ciphertext, one per prime.
//   x = REDC_p2(ct_mont) = c*Rp mod p^2;  y = x^(p-1) (sliding windows,
//   shared exponent program);  y = REDC(y);  then one lane finishes
//   L_p, CRT and the sign fold serially.
// ---------------------------------------------------------------------------
template <int H>
__device__ __noinline__ void s_montmul(uint32_t* r, const uint32_t* a, const uint32_t* b, const uint32_t* m, uint32_t np) {
  uint32_t t[H + 2];
#pragma unroll 1
  for (int i = 0; i < H + 2; ++i) t[i] = 0;
#pragma unroll 1
  for (int i = 0; i < H; ++i) {
    uint64_t c = 0;
    const uint32_t bi = b[i];
#pragma unroll 1
    for (int j = 0; j < H; ++j) {
      c += (uint64_t)a[j] * bi + t[j];
      t[j] = (uint32_t)c;
      c >>= 32;
    }
    c += t[H];
    t[H] = (uint32_t)c;
    t[H + 1] = (uint32_t)(c >> 32);
    const uint32_t mq = t[0] * np;
    c = ((uint64_t)mq * m[0] + t[0]) >> 32;
#pragma unroll 1
    for (int j = 1; j < H; ++j) {
      c += (uint64_t)mq * m[j] + t[j];
      t[j - 1] = (uint32_t)c;
      c >>= 32;
    }
    c += t[H];
    t[H - 1] = (uint32_t)c;
    t[H] = t[H + 1] + (uint32_t)(c >> 32);
  }
  // conditional subtract
  uint32_t d[H];
  int64_t br = 0;
#pragma unroll 1
  for (int j = 0; j < H; ++j) {
    const int64_t v = (int64_t)t[j] - m[j] - br;
    br = v < 0;
    d[j] = (uint32_t)v;
  }
  const bool take = (t[H] != 0) || (br == 0);
#pragma unroll 1
  for (int j = 0; j < H; ++j) r[j] = take ? d[j] : t[j];
}

// r = a - b (H limbs), returns borrow
template <int H>
__device__ __forceinline__ uint32_t s_sub(uint32_t* r, const uint32_t* a, const uint32_t* b) {
  int64_t br = 0;
#pragma unroll 1
  for (int j = 0; j < H; ++j) {
    const int64_t v = (int64_t)a[j] - b[j] - br;
    br = v < 0;
    r[j] = (uint32_t)v;
  }
  return (uint32_t)br;
}

template <int TP, int LP>
__global__ void __launch_bounds__(kBlock) k_decrypt(KeyConst kc, SecConst sc, const uint32_t* __restrict__ ct,
                                                    size_t count, int64_t* __restrict__ out_i64,
                                                    uint8_t* __restrict__ out_ovf, uint32_t* __restrict__ out_mag,
                                                    uint8_t* __restrict__ out_neg, uint32_t* __restrict__ scratch,
                                                    uint32_t* err) {
  constexpr int SP = TP * LP;   // limbs of p^2
  constexpr int H = SP / 2;     // limbs of p
  constexpr int UPW = 32 / (2 * TP);  // ciphertexts per warp
  constexpr int UPB = kBlock / (2 * TP);
  __shared__ __align__(16) uint32_t ysm[UPB][2][SP];
  const Group<TP> g;
  const int lane = threadIdx.x & 31;
  const int side = (lane / TP) & 1;
  const int unit_w = lane / (2 * TP);
  const int unit_b = threadIdx.x / (2 * TP);
  const int warp_first = (threadIdx.x >> 5) * UPW;
  const size_t stride = (size_t)gridDim.x * UPB;
  const int ntab = 1 << (sc.wd - 1);
  uint32_t* tb = scratch + (((size_t)blockIdx.x * UPB + unit_b) * 2 + side) * (size_t)ntab * SP + g.t * LP;
  uint32_t N[LP];
  load_slice<LP>(N, sc.P2[side] + g.t * LP);
  const uint32_t np = sc.np2[side];
  const uint16_t* prog = sc.prog[side];
  for (size_t wbase = (size_t)blockIdx.x * UPB + warp_first; wbase < count; wbase += stride) {
    const size_t inst = wbase + unit_w;
    const bool active = inst < count;
    const size_t i = active ? inst : count - 1;
    uint32_t lo[LP], hi[LP], x[LP];
    load_slice<LP>(lo, ct + i * (2 * SP) + g.t * LP);
    load_slice<LP>(hi, ct + i * (2 * SP) + SP + g.t * LP);
    {
      // validate against n^2 (decryptor.cc:21-23): the p side holds the low
      // half; compare the whole number with a lookahead over both halves.
      uint32_t Nlo[LP], Nhi[LP], d[LP];
      load_slice<LP>(Nlo, kc.N + g.t * LP);
      load_slice<LP>(Nhi, kc.N + SP + g.t * LP);
      const uint32_t b_lo = sub_full<TP, LP>(d, lo, Nlo, g);
      // hi - Nhi - b_lo: borrow out means ct < N
      uint32_t e2[LP];
      (void)sub_full<TP, LP>(e2, hi, Nhi, g);
      const bool hi_lt = less_than<TP, LP>(hi, Nhi, g);
      const bool hi_eq = is_zero<TP, LP>(e2, g);
      const bool ok = hi_lt || (hi_eq && b_lo);
      if (active && !ok && g.t == 0 && side == 0) atomicOr(err, kErrCtRange);
    }
    mont_redc_wide<TP, LP>(x, lo, hi, N, np, g);
    // odd powers x, x^3, ...
    store_slice<LP>(tb, x);
    uint32_t x2[LP], cur[LP];
    mont_mul<TP, LP>(x2, x, x, N, np, g);
    copy_slice<LP>(cur, x);
#pragma unroll 1
    for (int t = 1; t < ntab; ++t) {
      mont_mul<TP, LP>(cur, cur, x2, N, np, g);
      store_slice<LP>(tb + (size_t)t * SP, cur);
    }
    uint32_t acc[LP];
    load_slice<LP>(acc, tb + (size_t)sc.start[side] * SP);
#pragma unroll 1
    for (int s = 0; s < sc.prog_len; ++s) {
      const uint16_t op = prog[s];
      uint32_t B[LP];
      if (op < kOpNop) {
        load_slice<LP>(B, tb + (size_t)op * SP);
      } else {
        copy_slice<LP>(B, acc);
      }
      uint32_t res[LP];
      mont_mul<TP, LP>(res, acc, B, N, np, g);
      if (op != kOpNop) copy_slice<LP>(acc, res);
    }
    mont_redc<TP, LP>(acc, acc, N, np, g);
    // hand both halves to one lane
#pragma unroll
    for (int j = 0; j < LP; ++j) ysm[unit_b][side][g.t * LP + j] = acc[j];
    __syncwarp();
    if (side == 0 && g.t == 0) {
      uint32_t Lv[H], mp[H], mq[H], t1[H];
      // L_p = (y_p - 1)/p exactly = ((y_p - 1) mod 2^(32H)) * p^-1 mod 2^(32H)
#pragma unroll 1
      #pragma unroll 1
      for (int sd = 0; sd < 2; ++sd) {
        const uint32_t* y = ysm[unit_b][sd];
        uint64_t br = 1;
        #pragma unroll 1
        for (int j = 0; j < H; ++j) {
          const uint64_t v = (uint64_t)y[j] - br;
          t1[j] = (uint32_t)v;
          br = (v >> 63) & 1ull;
        }
        const uint32_t* iv = sc.inv2[sd];
        #pragma unroll 1
        for (int j = 0; j < H; ++j) Lv[j] = 0;
        #pragma unroll 1
        for (int a = 0; a < H; ++a) {
          uint64_t c = 0;
          const uint32_t ta = t1[a];
          #pragma unroll 1
          for (int b = 0; a + b < H; ++b) {
            c += (uint64_t)ta * iv[b] + Lv[a + b];
            Lv[a + b] = (uint32_t)c;
            c >>= 32;
          }
        }
        s_montmul<H>(sd == 0 ? mp : mq, Lv, sc.hR[sd], sc.P[sd], sc.np1[sd]);
      }
      // mp mod q (p < 2q), d = mq - mp mod q, h = d * p^-1 mod q
      const uint32_t* Q = sc.P[1];
      uint32_t mpq[H];
      {
        const uint32_t b = s_sub<H>(t1, mp, Q);
        #pragma unroll 1
        for (int j = 0; j < H; ++j) mpq[j] = b ? mp[j] : t1[j];
      }
      uint32_t dd[H];
      {
        const uint32_t b = s_sub<H>(dd, mq, mpq);
        if (b) {
          uint64_t c = 0;
          #pragma unroll 1
          for (int j = 0; j < H; ++j) {
            c += (uint64_t)dd[j] + Q[j];
            dd[j] = (uint32_t)c;
            c >>= 32;
          }
        }
      }
      uint32_t hh[H];
      s_montmul<H>(hh, dd, sc.pinvqR, Q, sc.np1[1]);
      // m = mp + p*h  (2H limbs)
      uint32_t mm[2 * H];
      const uint32_t* P = sc.P[0];
      #pragma unroll 1
      for (int j = 0; j < 2 * H; ++j) mm[j] = j < H ? mp[j] : 0u;
      #pragma unroll 1
      for (int a = 0; a < H; ++a) {
        uint64_t c = 0;
        const uint32_t pa = P[a];
        #pragma unroll 1
        for (int b = 0; b < H; ++b) {
          c += (uint64_t)pa * hh[b] + mm[a + b];
          mm[a + b] = (uint32_t)c;
          c >>= 32;
        }
        #pragma unroll 1
        for (int j = a + H; c && j < 2 * H; ++j) {
          c += mm[j];
          mm[j] = (uint32_t)c;
          c >>= 32;
        }
      }
      // sign fold: m > n/2 => m - n (decryptor.cc:49-52)
      bool gt = false;
      #pragma unroll 1
      for (int j = 2 * H - 1; j >= 0; --j) {
        const uint32_t hv = kc.nhalf[j];
        if (mm[j] != hv) {
          gt = mm[j] > hv;
          break;
        }
      }
      if (gt) {
        // magnitude = n - m
        int64_t br = 0;
        #pragma unroll 1
        for (int j = 0; j < 2 * H; ++j) {
          const int64_t v = (int64_t)kc.n[j] - mm[j] - br;
          br = v < 0;
          mm[j] = (uint32_t)v;
        }
      }
      if (active) {
        if (out_mag) {
          #pragma unroll 1
          for (int j = 0; j < 2 * H; ++j) out_mag[i * (2 * H) + j] = mm[j];
          out_neg[i] = gt ? 1 : 0;
        }
        if (out_i64) {
          bool fits = true;
          #pragma unroll 1
          for (int j = 2; j < 2 * H; ++j) fits &= (mm[j] == 0u);
          const uint64_t mag = (uint64_t)mm[0] | ((uint64_t)mm[1] << 32);
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
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Montgomery conversion: to_mont = MM(x, R^2), from_mont = REDC(x)
// ---------------------------------------------------------------------------
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_convert(KeyConst kc, const uint32_t* __restrict__ in,
                                                    uint32_t* __restrict__ out, size_t count, int to_mont,
                                                    uint32_t* err) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  if (wfirst >= count) return;
  const bool active = inst < count;
  const size_t i = active ? inst : count - 1;
  uint32_t N[L], A[L], B[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(A, in + i * S + g.t * L);
  check_ct<TPI, L>(A, N, active, g, err);
  if (to_mont) {
    load_slice<L>(B, kc.R2 + g.t * L);
    mont_mul<TPI, L>(A, A, B, N, kc.np, g);
  } else {
    mont_redc<TPI, L>(A, A, N, kc.np, g);
  }
  if (active) store_slice<L>(out + i * S + g.t * L, A);
}

// ---------------------------------------------------------------------------
// Chunked product reduction: out[j] = prod in[j*chunk .. (j+1)*chunk)
// (numpy/evaluator.cc:355-373 reduces with AddInplace = MulMod)
// ---------------------------------------------------------------------------
template <int TPI, int L>
__global__ void __launch_bounds__(kBlock) k_reduce(KeyConst kc, const uint32_t* __restrict__ in, size_t count,
                                                   int chunk, uint32_t* __restrict__ out, size_t out_count,
                                                   uint32_t* err) {
  constexpr int S = TPI * L;
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  if (wfirst >= out_count) return;
  const bool active = inst < out_count;
  const size_t o = active ? inst : out_count - 1;
  uint32_t N[L], acc[L];
  load_slice<L>(N, kc.N + g.t * L);
  const size_t first = o * (size_t)chunk;
  load_slice<L>(acc, in + first * S + g.t * L);
  check_ct<TPI, L>(acc, N, active, g, err);
#pragma unroll 1
  for (int j = 1; j < chunk; ++j) {
    const size_t idx = first + j;
    const bool valid = idx < count;
    if (!__any_sync(kFull, valid)) break;
    uint32_t B[L];
    load_slice<L>(B, (valid ? in + idx * S : kc.R1) + g.t * L);
    mont_mul<TPI, L>(acc, acc, B, N, kc.np, g);
  }
  if (active) store_slice<L>(out + o * S + g.t * L, acc);
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
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  if (wfirst >= upper_count) return;
  const bool active = inst < upper_count;
  const size_t i = active ? inst : upper_count - 1;
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
  const Group<TPI> g;
  const size_t inst = ((size_t)blockIdx.x * kBlock + threadIdx.x) / TPI;
  const size_t wfirst = ((size_t)blockIdx.x * kBlock + (threadIdx.x & ~31u)) / TPI;
  if (wfirst >= upper_count) return;
  const bool active = inst < upper_count;
  const size_t i = active ? inst : upper_count - 1;
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

// root_slot = MM(z, R^3) where z = (X*R)^-1 mod N, giving X^-1 * R.
template <int TPI, int L>
__global__ void __launch_bounds__(32) k_root_fix(KeyConst kc, const uint32_t* __restrict__ z,
                                                 uint32_t* __restrict__ root_slot) {
  const Group<TPI> g;
  uint32_t N[L], A[L], B[L];
  load_slice<L>(N, kc.N + g.t * L);
  load_slice<L>(A, z + g.t * L);
  load_slice<L>(B, kc.R3 + g.t * L);
  mont_mul<TPI, L>(A, A, B, N, kc.np, g);
  if (threadIdx.x < TPI) store_slice<L>(root_slot + g.t * L, A);
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
// variant selection: (limbs) -> (threads per instance, limbs per thread)
// ---------------------------------------------------------------------------
#define HG_DISPATCH_S(S, ...)                                \
  switch (S) {                                               \
    case 64: { constexpr int TPI = 4, L = 16; __VA_ARGS__; } break;  \
    case 128: { constexpr int TPI = 8, L = 16; __VA_ARGS__; } break; \
    case 192: { constexpr int TPI = 16, L = 12; __VA_ARGS__; } break; \
    default: return cudaErrorInvalidValue;                   \
  }

#define HG_DISPATCH_SP(SP, ...)                              \
  switch (SP) {                                              \
    case 32: { constexpr int TP = 2, LP = 16; __VA_ARGS__; } break;  \
    case 64: { constexpr int TP = 4, LP = 16; __VA_ARGS__; } break;  \
    case 96: { constexpr int TP = 8, LP = 12; __VA_ARGS__; } break;  \
    default: return cudaErrorInvalidValue;                   \
  }

bool supported_limbs(int S) { return S == 64 || S == 128 || S == 192; }

static std::atomic<uint64_t> g_launches{0};
uint64_t launch_count() { return g_launches.load(); }
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

int instances_per_block(int S) {
  switch (S) {
    case 64: return kBlock / 4;
    case 128: return kBlock / 8;
    case 192: return kBlock / 16;
    default: return 0;
  }
}
int units_per_block_decrypt(int Sp) {
  switch (Sp) {
    case 32: return kBlock / 4;
    case 64: return kBlock / 8;
    case 96: return kBlock / 16;
    default: return 0;
  }
}

int resident_blocks_encrypt(int S) {
  int r = 0;
  [&]() -> cudaError_t { HG_DISPATCH_S(S, r = occupancy_blocks(k_encrypt<TPI, L>)); return cudaSuccess; }();
  return r;
}
int resident_blocks_mul(int S) {
  int r = 0;
  [&]() -> cudaError_t { HG_DISPATCH_S(S, r = occupancy_blocks(k_mul<TPI, L>)); return cudaSuccess; }();
  return r;
}
int resident_blocks_decrypt(int Sp) {
  int r = 0;
  [&]() -> cudaError_t { HG_DISPATCH_SP(Sp, r = occupancy_blocks(k_decrypt<TP, LP>)); return cudaSuccess; }();
  return r;
}

cudaError_t launch_encrypt(int S, const KeyConst& kc, EncMode mode, const int64_t* m, const uint32_t* m_mag,
                           const uint8_t* m_neg, const uint32_t* r, const uint32_t* ct_in, uint32_t* out,
                           size_t count, uint32_t* err, int grid, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  HG_DISPATCH_S(S, {
    const unsigned need = blocks_for(count, TPI);
    const unsigned gb = (unsigned)std::min((size_t)need, (size_t)(grid > 0 ? (unsigned)grid : need));
    k_encrypt<TPI, L><<<gb, kBlock, 0, st>>>(kc, mode, m, m_mag, m_neg, r, ct_in, out, count, err);
  });
  return counted();
}

cudaError_t launch_add(int S, const KeyConst& kc, const uint32_t* a, const uint32_t* b, uint32_t* out,
                       size_t count, uint32_t* err, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  HG_DISPATCH_S(S, k_add<TPI, L><<<blocks_for(count, TPI), kBlock, 0, st>>>(kc, a, b, out, count, err));
  return counted();
}

cudaError_t launch_add_plain(int S, const KeyConst& kc, const uint32_t* a, const int64_t* p, int neg_p,
                             uint32_t* out, size_t count, uint32_t* err, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  HG_DISPATCH_S(S, k_add_plain<TPI, L><<<blocks_for(count, TPI), kBlock, 0, st>>>(kc, a, p, neg_p, out,
                                                                                   count, err));
  return counted();
}

cudaError_t launch_mul(int S, const KeyConst& kc, const uint32_t* a, const int64_t* k, uint32_t* out,
                       size_t count, uint32_t* scratch, int wm, uint32_t* err, int grid, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  HG_DISPATCH_S(S, {
    const unsigned need = blocks_for(count, TPI);
    const unsigned gb = (unsigned)std::min((size_t)need, (size_t)grid);
    k_mul<TPI, L><<<gb, kBlock, 0, st>>>(kc, a, k, out, count, scratch, wm, err);
  });
  return counted();
}

cudaError_t launch_decrypt(int Sp, const KeyConst& kc, const SecConst& sc, const uint32_t* ct, size_t count,
                           int64_t* out_i64, uint8_t* out_ovf, uint32_t* out_mag, uint8_t* out_neg,
                           uint32_t* scratch, uint32_t* err, int grid, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  HG_DISPATCH_SP(Sp, {
    const size_t upb = kBlock / (2 * TP);
    const unsigned need = (unsigned)((count + upb - 1) / upb);
    const unsigned gb = (unsigned)std::min((size_t)need, (size_t)grid);
    k_decrypt<TP, LP><<<gb, kBlock, 0, st>>>(kc, sc, ct, count, out_i64, out_ovf, out_mag, out_neg, scratch,
                                              err);
  });
  return counted();
}

cudaError_t launch_convert(int S, const KeyConst& kc, const uint32_t* in, uint32_t* out, size_t count,
                           int to_mont, uint32_t* err, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  HG_DISPATCH_S(S, k_convert<TPI, L><<<blocks_for(count, TPI), kBlock, 0, st>>>(kc, in, out, count, to_mont,
                                                                                 err));
  return counted();
}

cudaError_t launch_reduce(int S, const KeyConst& kc, const uint32_t* in, size_t count, int chunk,
                          uint32_t* out, uint32_t* err, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  const size_t out_count = (count + chunk - 1) / chunk;
  HG_DISPATCH_S(S, k_reduce<TPI, L><<<blocks_for(out_count, TPI), kBlock, 0, st>>>(kc, in, count, chunk, out,
                                                                                    out_count, err));
  return counted();
}

cudaError_t launch_tree_leaves(int S, const KeyConst& kc, const uint32_t* in, const int64_t* sel, size_t count,
                               uint32_t* leaves, size_t padded, uint32_t* err, cudaStream_t st) {
  HG_DISPATCH_S(S, k_tree_leaves<TPI, L><<<blocks_for(padded, TPI), kBlock, 0, st>>>(kc, in, sel, count,
                                                                                      leaves, padded, err));
  return counted();
}

cudaError_t launch_tree_up(int S, const KeyConst& kc, const uint32_t* lower, uint32_t* upper, size_t upper_count,
                           cudaStream_t st) {
  HG_DISPATCH_S(S, k_tree_up<TPI, L><<<blocks_for(upper_count, TPI), kBlock, 0, st>>>(kc, lower, upper,
                                                                                       upper_count));
  return counted();
}

cudaError_t launch_tree_down(int S, const KeyConst& kc, uint32_t* lower, const uint32_t* upper_inv,
                             size_t upper_count, cudaStream_t st) {
  HG_DISPATCH_S(S, k_tree_down<TPI, L><<<blocks_for(upper_count, TPI), kBlock, 0, st>>>(kc, lower, upper_inv,
                                                                                         upper_count));
  return counted();
}

cudaError_t launch_tree_apply(int S, const KeyConst& kc, const uint32_t* in, const int64_t* sel,
                              const uint32_t* leaves_inv, uint32_t* out, size_t count, cudaStream_t st) {
  HG_DISPATCH_S(S, k_tree_apply<TPI, L><<<blocks_for(count, TPI), kBlock, 0, st>>>(kc, in, sel, leaves_inv,
                                                                                    out, count));
  return counted();
}

cudaError_t launch_root_fix(int S, const KeyConst& kc, const uint32_t* root_inv_z, uint32_t* root_slot,
                            cudaStream_t st) {
  HG_DISPATCH_S(S, k_root_fix<TPI, L><<<1, 32, 0, st>>>(kc, root_inv_z, root_slot));
  return counted();
}

cudaError_t launch_table_bases(int S, const KeyConst& kc, const uint32_t* hs_mont, uint32_t* bases,
                               cudaStream_t st) {
  HG_DISPATCH_S(S, k_table_bases<TPI, L><<<1, 32, 0, st>>>(kc, hs_mont, bases));
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
  HG_DISPATCH_S(S, k_table_level<TPI, L><<<blocks_for(total, TPI), kBlock, 0, st>>>(kc, table, bases, level));
  return counted();
}

}  // namespace hg

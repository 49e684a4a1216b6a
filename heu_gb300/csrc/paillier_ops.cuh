// Per-ciphertext operation bodies shared by the standalone kernels
// (paillier_kernels.cu, decrypt_kernels.cu) and the persistent multi-key
// batch kernel (batch_kernels.cu).
//
// Every *_one function processes one ciphertext per group of lanes: the
// caller passes the clamped instance index `i` and whether it is `active`;
// all groups of a warp call the same function together (full-warp shuffles
// and ballots inside).
#pragma once
#include "mont.cuh"
#include "paillier_kernels.cuh"

namespace hg {

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

// 32 bits at bit offset 32*gi of (u << sh), for any sh >= 0.
__device__ __forceinline__ uint32_t limb_of_shifted(uint64_t u, int sh, int gi) {
  const int off = 32 * gi - sh;
  if (off >= 64 || off <= -32) return 0u;
  return off >= 0 ? (uint32_t)(u >> off) : (uint32_t)(u << (-off));
}

// The plaintext of element i under a device encoding, as the pieces from
// which its magnitude's limbs are cut: magnitude = lo + (hi << hsh) (hi may
// be 0), sign `neg`; `bad` when the value cannot be encoded (non-finite or
// out-of-range doubles).
//   PlainEncoder (plain_encoder.h:58-61): int64 x -> int128(x) * scale;
//     double x -> trunc(x * scale) as an integer of any size.
//   BatchEncoder (batch_encoder.h:53-80, 119-126): the 64-bit two's
//     complement patterns of a * scale and b * scale (doubles: int64(trunc(
//     x * scale))), b's shifted up by 64 + padding bits.
struct EncodedPlain {
  uint64_t lo = 0, hi = 0;
  int hsh = 64;
  bool neg = false, bad = false;
};

__device__ __forceinline__ EncodedPlain encode_plain(const Codec& cd, const int64_t* __restrict__ m, size_t i) {
  EncodedPlain e;
  const double sc = (double)cd.scale;
  switch (cd.kind) {
    case kCodecPlainI64: {
      const int64_t x = m[i];
      const uint64_t a = x < 0 ? (uint64_t)0 - (uint64_t)x : (uint64_t)x;
      const uint64_t s = (uint64_t)cd.scale;
      e.lo = a * s;
      e.hi = __umul64hi(a, s);
      e.neg = x < 0 && a != 0;
      break;
    }
    case kCodecPlainF64: {
      const double d = trunc(reinterpret_cast<const double*>(m)[i] * sc);
      if (!isfinite(d)) {
        e.bad = true;
        break;
      }
      e.neg = d < 0.0;
      const double a = fabs(d);
      if (a < 18446744073709551616.0) {
        e.lo = (uint64_t)a;
      } else {  // a = mantissa * 2^ex exactly (integer-valued, ex >= 12)
        const uint64_t bits = (uint64_t)__double_as_longlong(a);
        const int ex = (int)((bits >> 52) & 0x7ff) - 1075;
        e.hi = (bits & ((1ull << 52) - 1)) | (1ull << 52);
        e.hsh = ex;
      }
      break;
    }
    case kCodecBatchI64:
    case kCodecBatchF64: {
      int64_t a, b;
      if (cd.kind == kCodecBatchI64) {
        a = (int64_t)((uint64_t)m[i] * (uint64_t)cd.scale);
        b = (int64_t)((uint64_t)reinterpret_cast<const int64_t*>(cd.in1)[i] * (uint64_t)cd.scale);
      } else {
        const double da = trunc(reinterpret_cast<const double*>(m)[i] * sc);
        const double db = trunc(reinterpret_cast<const double*>(cd.in1)[i] * sc);
        // static_cast<int64_t>(double) needs the value in int64's range
        const double lim = 9223372036854775808.0;
        if (!(da >= -lim && da < lim && db >= -lim && db < lim)) {
          e.bad = true;
          break;
        }
        a = (int64_t)da;
        b = (int64_t)db;
      }
      e.lo = (uint64_t)a;
      e.hi = (uint64_t)b;
      e.hsh = 64 + cd.padding;
      break;
    }
    default:
      break;
  }
  return e;
}

__device__ __forceinline__ uint32_t encoded_limb(const EncodedPlain& e, int gi) {
  return limb_of_shifted(e.lo, 0, gi) | limb_of_shifted(e.hi, e.hsh, gi);
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
// Encrypt / EncryptZero / Randomize (encryptor.cc:26-56, evaluator.cc:25-28):
//   acc = gm(m) | R | ct_in;  acc *= prod_pos table[pos][digit_pos(r)]
// ---------------------------------------------------------------------------
template <int TPI, int L>
__device__ __forceinline__ void encrypt_one(const KeyConst& kc, EncMode mode, const int64_t* __restrict__ m,
                                            const uint32_t* __restrict__ m_mag, const uint8_t* __restrict__ m_neg,
                                            const uint32_t* __restrict__ r, const uint32_t* __restrict__ ct_in,
                                            uint32_t* __restrict__ out, size_t i, bool active,
                                            const uint32_t (&N)[L], const Group<TPI>& g, uint32_t* err,
                                            const Codec& cd = Codec{}) {
  constexpr int S = TPI * L;
  uint32_t acc[L];
  if (mode == EncMode::kEncrypt) {
    uint32_t A[L];
    bool neg;
    if (cd.kind != kCodecNone) {
      // encoded on the device; |m| <= n/2 as for any plaintext (encryptor.cc:38-40)
      const EncodedPlain e = encode_plain(cd, m, i);
      uint32_t NH[L], d[L];
#pragma unroll
      for (int j = 0; j < L; ++j) {
        const int gi = (int)g.t * L + j;
        A[j] = gi < S / 2 ? encoded_limb(e, gi) : 0u;
        NH[j] = gi < S / 2 ? kc.nhalf[gi] : 0u;
      }
      neg = e.neg;
      const bool too_big = sub_full<TPI, L>(d, NH, A, g) != 0u;
      if (active && (too_big || e.bad) && g.t == 0) atomicOr(err, kErrPtRange);
      // a value that does not fit is replaced by 0 (its error is reported)
      if (too_big || e.bad) {
#pragma unroll
        for (int j = 0; j < L; ++j) A[j] = 0u;
      }
    } else if (m_mag != nullptr) {
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
  const size_t ent = (size_t)((1u << kc.w) - 1u);
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

// Add(ct, ct): MulMod of Montgomery residues (evaluator.cc:30-44)
template <int TPI, int L>
__device__ __forceinline__ void add_one(const KeyConst& kc, const uint32_t* __restrict__ a,
                                        const uint32_t* __restrict__ b, uint32_t* __restrict__ out, size_t i,
                                        bool active, const uint32_t (&N)[L], const Group<TPI>& g, uint32_t* err) {
  constexpr int S = TPI * L;
  uint32_t A[L], B[L];
  load_slice<L>(A, a + i * S + g.t * L);
  load_slice<L>(B, b + i * S + g.t * L);
  check_ct<TPI, L>(A, N, active, g, err);
  check_ct<TPI, L>(B, N, active, g, err);
  mont_mul<TPI, L>(A, A, B, N, kc.np, g);
  if (active) store_slice<L>(out + i * S + g.t * L, A);
}

// Add(ct, pt) / Sub(ct, pt): a * (1 + n*p) (evaluator.cc:46-76)
template <int TPI, int L>
__device__ __forceinline__ void add_plain_one(const KeyConst& kc, const uint32_t* __restrict__ a,
                                              const int64_t* __restrict__ p, int neg_p, uint32_t* __restrict__ out,
                                              size_t i, bool active, const uint32_t (&N)[L], const Group<TPI>& g,
                                              uint32_t* err) {
  constexpr int S = TPI * L;
  uint32_t A[L], G[L], Am[L];
  load_slice<L>(A, a + i * S + g.t * L);
  check_ct<TPI, L>(A, N, active, g, err);
  const int64_t pv = p[i];
  // Sub(ct, pt) adds -p (evaluator.cc:74-76); the magnitude covers INT64_MIN
  set_u64<TPI, L>(Am, g, abs_i64(pv));
  to_gm<TPI, L>(G, Am, (pv < 0) != (neg_p != 0), N, kc, g);
  mont_mul<TPI, L>(A, A, G, N, kc.np, g);
  if (active) store_slice<L>(out + i * S + g.t * L, A);
}

// Mul(ct, k) for 64-bit k: c^|k| by left-to-right sliding windows (odd powers
// c, c^3, .., c^(2^wm - 1) in this group's table `tb`, already offset by the
// lane's slice).  k = 0 gives the Montgomery identity (evaluator.cc:105-106);
// k < 0 is finished by a batch inverse afterwards (evaluator.cc:119-121).
// Every step is one Montgomery multiplication for every group of the warp;
// only the operand differs (square, table entry, or a discarded step).
template <int TPI, int L>
__device__ __forceinline__ void mul_one(const KeyConst& kc, const uint32_t* __restrict__ a,
                                        const int64_t* __restrict__ kk, uint32_t* __restrict__ out, size_t i,
                                        bool active, uint32_t* __restrict__ tb, int wm, const uint32_t (&N)[L],
                                        const Group<TPI>& g, uint32_t* err) {
  constexpr int S = TPI * L;
  const int ntab = 1 << (wm - 1);
  const uint64_t e = abs_i64(kk[i]);
  uint32_t x[L];
  load_slice<L>(x, a + i * S + g.t * L);
  check_ct<TPI, L>(x, N, active, g, err);
  store_slice<L>(tb, x);
  uint32_t x2[L], cur[L];
  mont_mul<TPI, L>(x2, x, x, N, kc.np, g);
  copy_slice<L>(cur, x);
#pragma unroll 1
  for (int t = 1; t < ntab; ++t) {
    mont_mul<TPI, L>(cur, cur, x2, N, kc.np, g);
    store_slice<L>(tb + (size_t)t * S, cur);
  }
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

// Mul(ct, k) for a scalar of any size up to `el` 32-bit limbs (magnitude in
// `emag`, little-endian; the sign is applied afterwards by the batch
// inverse).  evaluator.cc:99-123 takes any BigInt ("ciphertext overflow is
// allowed"): c^|k| mod n^2 by left-to-right sliding windows of `wb` bits over
// the limbs, odd powers c, c^3, .., c^(2^wb - 1) in this group's table `tb`.
// |k| = 0 gives the Montgomery identity (evaluator.cc:105-106).
template <int TPI, int L>
__device__ __forceinline__ void mul_bn_one(const KeyConst& kc, const uint32_t* __restrict__ a,
                                           const uint32_t* __restrict__ emag, int el, uint32_t* __restrict__ out,
                                           size_t i, bool active, uint32_t* __restrict__ tb, int wb,
                                           const uint32_t (&N)[L], const Group<TPI>& g, uint32_t* err) {
  constexpr int S = TPI * L;
  const int ntab = 1 << (wb - 1);
  const uint32_t* e = emag + i * (size_t)el;
  int pos = -1;
#pragma unroll 1
  for (int l = el - 1; l >= 0; --l) {
    const uint32_t v = e[l];
    if (v != 0u) {
      pos = l * 32 + 31 - __clz(v);
      break;
    }
  }
  uint32_t x[L];
  load_slice<L>(x, a + i * S + g.t * L);
  check_ct<TPI, L>(x, N, active, g, err);
  store_slice<L>(tb, x);
  uint32_t x2[L], cur[L];
  mont_mul<TPI, L>(x2, x, x, N, kc.np, g);
  copy_slice<L>(cur, x);
#pragma unroll 1
  for (int t = 1; t < ntab; ++t) {
    mont_mul<TPI, L>(cur, cur, x2, N, kc.np, g);
    store_slice<L>(tb + (size_t)t * S, cur);
  }
  // the window ending at bit `top`: its lowest set bit j and its value
  auto window = [&](int top, int& j) -> uint32_t {
    j = max(top - wb + 1, 0);
    while (!((e[j >> 5] >> (j & 31)) & 1u)) ++j;
    return get_bits(e, el, j, top - j + 1);
  };
  uint32_t acc[L];
  int sq = 0, mulidx = -1;
  if (pos >= 0) {
    int j;
    const uint32_t val = window(pos, j);
    load_slice<L>(acc, tb + (size_t)((val - 1) >> 1) * S);
    pos = j - 1;
  } else {
    load_slice<L>(acc, kc.R1 + g.t * L);
  }
#pragma unroll 1
  while (true) {
    int op = 0;  // 0 = none, 1 = square, 2 = multiply by table[mulidx]
    if (sq > 0) {
      op = 1;
      --sq;
    } else if (mulidx >= 0) {
      op = 2;
    } else if (pos >= 0) {
      if (!((e[pos >> 5] >> (pos & 31)) & 1u)) {
        op = 1;
        --pos;
      } else {
        int j;
        const uint32_t val = window(pos, j);
        sq = pos - j;
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

// ---------------------------------------------------------------------------
// Decrypt (decryptor.cc:32-53): two groups per ciphertext, one per prime.
//   x = REDC_p2(ct_mont) = c*Rp mod p^2;  y = x^(p-1) (sliding windows,
//   shared exponent program);  y = REDC(y);  then one lane finishes
//   L_p, CRT and the sign fold serially.
// ---------------------------------------------------------------------------
template <int H>
__device__ __noinline__ void s_montmul(uint32_t* r, const uint32_t* a, const uint32_t* b, const uint32_t* m,
                                       uint32_t np) {
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

// Serial CRT tail for one ciphertext, run by one lane: y[0], y[1] = the
// Z-form values c^(p-1) mod p^2 and c^(q-1) mod q^2 (SP = 2H limbs each).
// Decoding of a decrypted plaintext (magnitude mm of W limbs, negative when
// `neg`) under a device encoding, into out0 / cd.out1 (element i) and the
// overflow flag:
//   PlainEncoder::Decode (plain_encoder.h:64-69): int64 -> m / scale with
//     C++ division (toward zero), flagged when it does not fit int64;
//     double -> double(m) rounded to nearest-even, / scale (flagged, +-inf,
//     beyond the double range).
//   BatchEncoder::Decode (batch_encoder.h:85-103): slot s = the low 64 bits
//     of m >> s * (64 + padding) as int64 (the sign of m applied as BigInt
//     shifts and GetValue do: on the magnitude), / scale (int64 division, or
//     double division for the double kind); flagged when m < 0.
template <int W>
__device__ void decode_plain(const Codec& cd, const uint32_t* mm, bool neg, size_t i, void* out0, uint8_t* ovf) {
  if (cd.kind == kCodecPlainI64) {
    bool wide = false;
#pragma unroll 1
    for (int j = 4; j < W; ++j) wide |= mm[j] != 0u;
    const unsigned __int128 mag = (unsigned __int128)((uint64_t)mm[0] | ((uint64_t)mm[1] << 32)) |
                                  ((unsigned __int128)((uint64_t)mm[2] | ((uint64_t)mm[3] << 32)) << 64);
    const unsigned __int128 q = mag / (unsigned __int128)(uint64_t)cd.scale;
    const bool fits = !wide && (q < ((unsigned __int128)1 << 63) || (neg && q == ((unsigned __int128)1 << 63)));
    const uint64_t q64 = (uint64_t)q;
    reinterpret_cast<int64_t*>(out0)[i] = fits ? (int64_t)(neg ? (uint64_t)0 - q64 : q64) : 0;
    if (ovf) ovf[i] = fits ? 0 : 1;
    return;
  }
  if (cd.kind == kCodecPlainF64) {
    int top = -1;
#pragma unroll 1
    for (int j = W - 1; j >= 0 && top < 0; --j)
      if (mm[j] != 0u) top = j;
    double d = 0.0;
    if (top >= 0) {
      const int p = 32 * top + 31 - __clz(mm[top]);  // position of the top bit
      if (p < 64) {
        d = __ull2double_rn((uint64_t)mm[0] | ((uint64_t)(W > 1 ? mm[1] : 0u) << 32));
      } else {
        // the 64 bits below and including the top bit, the rest as a sticky bit
        const int lo = p - 63;
        uint64_t v = 0;
#pragma unroll 1
        for (int j = 0; j < W; ++j) {
          const int off = 32 * j - lo;  // bit position of limb j inside v
          if (off >= 64 || off <= -32) continue;
          v |= off >= 0 ? ((uint64_t)mm[j] << off) : ((uint64_t)mm[j] >> (-off));
        }
        bool sticky = false;
#pragma unroll 1
        for (int j = 0; j < W && 32 * j < lo; ++j) {
          const int keep = lo - 32 * j;  // bits of limb j below lo
          const uint32_t below = keep >= 32 ? mm[j] : (mm[j] & ((1u << keep) - 1u));
          sticky |= below != 0u;
        }
        d = ldexp(__ull2double_rn(v | (sticky ? 1ull : 0ull)), lo);
      }
    }
    d = neg ? -d : d;
    reinterpret_cast<double*>(out0)[i] = __ddiv_rn(d, (double)cd.scale);
    if (ovf) ovf[i] = isinf(d) ? 1 : 0;
    return;
  }
  // batch kinds: two slots
#pragma unroll 1
  for (int slot = 0; slot < 2; ++slot) {
    const int sh = slot * (64 + cd.padding);
    uint64_t v = 0;
#pragma unroll 1
    for (int j = 0; j < W; ++j) {
      const int off = 32 * j - sh;
      if (off >= 64 || off <= -32) continue;
      v |= off >= 0 ? ((uint64_t)mm[j] << off) : ((uint64_t)mm[j] >> (-off));
    }
    const int64_t x = neg ? (int64_t)((uint64_t)0 - v) : (int64_t)v;
    void* dst = slot == 0 ? out0 : cd.out1;
    if (cd.kind == kCodecBatchI64) {
      // C++ int64 division truncates toward zero
      const uint64_t a = x < 0 ? (uint64_t)0 - (uint64_t)x : (uint64_t)x;
      const uint64_t q = a / (uint64_t)cd.scale;
      reinterpret_cast<int64_t*>(dst)[i] = x < 0 ? (int64_t)((uint64_t)0 - q) : (int64_t)q;
    } else {
      reinterpret_cast<double*>(dst)[i] = __ddiv_rn((double)x, (double)cd.scale);
    }
  }
  // a negative packed plaintext means a slot underflowed its padding
  if (ovf) ovf[i] = neg ? 1 : 0;
}

template <int H>
__device__ __noinline__ void crt_tail(const KeyConst& kc, const SecConst& sc, const uint32_t* y0,
                                      const uint32_t* y1, size_t i, bool active, int64_t* __restrict__ out_i64,
                                      uint8_t* __restrict__ out_ovf, uint32_t* __restrict__ out_mag,
                                      uint8_t* __restrict__ out_neg, const Codec& cd) {
  uint32_t Lv[H], mp[H], mq[H], t1[H];
  // L_p = (y_p - 1)/p exactly = ((y_p - 1) mod 2^(32H)) * p^-1 mod 2^(32H)
#pragma unroll 1
  for (int sd = 0; sd < 2; ++sd) {
    const uint32_t* y = sd == 0 ? y0 : y1;
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
    int64_t br = 0;
#pragma unroll 1
    for (int j = 0; j < 2 * H; ++j) {
      const int64_t v = (int64_t)kc.n[j] - mm[j] - br;
      br = v < 0;
      mm[j] = (uint32_t)v;
    }
  }
  if (active && cd.kind != kCodecNone) {
    decode_plain<2 * H>(cd, mm, gt, i, out_i64, out_ovf);
    return;
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

// One ciphertext per pair of groups: `side` 0 works mod p^2, 1 mod q^2.
// `tb` is this group's odd-power table (offset by the lane's slice), `ysm`
// this ciphertext's hand-off buffer of 2 x SP limbs in shared memory.
template <int TP, int LP>
__device__ __forceinline__ void decrypt_one(const KeyConst& kc, const SecConst& sc, const uint32_t* __restrict__ ct,
                                            size_t i, bool active, int side, uint32_t* __restrict__ tb,
                                            uint32_t* ysm, int64_t* __restrict__ out_i64,
                                            uint8_t* __restrict__ out_ovf, uint32_t* __restrict__ out_mag,
                                            uint8_t* __restrict__ out_neg, const Group<TP>& g, uint32_t* err,
                                            const Codec& cd = Codec{}) {
  constexpr int SP = TP * LP;
  const int ntab = 1 << (sc.wd - 1);
  uint32_t N[LP];
  load_slice<LP>(N, sc.P2[side] + g.t * LP);
  const uint32_t np = sc.np2[side];
  const uint16_t* prog = sc.prog[side];
  uint32_t lo[LP], hi[LP], x[LP];
  load_slice<LP>(lo, ct + i * (2 * SP) + g.t * LP);
  load_slice<LP>(hi, ct + i * (2 * SP) + SP + g.t * LP);
  {
    // validate against n^2 (decryptor.cc:21-23)
    uint32_t Nlo[LP], Nhi[LP], d[LP];
    load_slice<LP>(Nlo, kc.N + g.t * LP);
    load_slice<LP>(Nhi, kc.N + SP + g.t * LP);
    const uint32_t b_lo = sub_full<TP, LP>(d, lo, Nlo, g);
    uint32_t e2[LP];
    (void)sub_full<TP, LP>(e2, hi, Nhi, g);
    const bool hi_lt = less_than<TP, LP>(hi, Nhi, g);
    const bool hi_eq = is_zero<TP, LP>(e2, g);
    const bool ok = hi_lt || (hi_eq && b_lo);
    if (active && !ok && g.t == 0 && side == 0) atomicOr(err, kErrCtRange);
  }
  mont_redc_wide<TP, LP>(x, lo, hi, N, np, g);
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
#pragma unroll
  for (int j = 0; j < LP; ++j) ysm[side * SP + g.t * LP + j] = acc[j];
  __syncwarp();
  if (side == 0 && g.t == 0)
    crt_tail<SP / 2>(kc, sc, ysm, ysm + SP, i, active, out_i64, out_ovf, out_mag, out_neg, cd);
  __syncwarp();
}

// Montgomery conversion: to_mont = MM(x, R^2), from_mont = REDC(x)
template <int TPI, int L>
__device__ __forceinline__ void convert_one(const KeyConst& kc, const uint32_t* __restrict__ in,
                                            uint32_t* __restrict__ out, int to_mont, size_t i, bool active,
                                            const uint32_t (&N)[L], const Group<TPI>& g, uint32_t* err) {
  constexpr int S = TPI * L;
  uint32_t A[L], B[L];
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

// The next `per_warp` work items for the calling warp, from a launch-wide
// counter zeroed before the launch.  Persistent kernels take their work this
// way rather than in fixed strided shares, so warps on faster SMs take more
// and none idles while another still holds a static share.
__device__ __forceinline__ size_t next_work(unsigned long long* ctr, int per_warp) {
  unsigned long long v = 0;
  if ((threadIdx.x & 31) == 0) v = atomicAdd(ctr, (unsigned long long)per_warp);
  return (size_t)__shfl_sync(0xffffffffu, v, 0);
}

}  // namespace hg

// ---------------------------------------------------------------------------
// (limbs, variant) -> (threads per instance, limbs per thread).  Variant 0 is
// the default; variant 1 is the alternative the autotuner may pick.
// ---------------------------------------------------------------------------
#define HG_DISPATCH_SV(S, V, ...)                                                        \
  switch ((S) * 2 + ((V) ? 1 : 0)) {                                                     \
    case 128: { constexpr int TPI = 4, L = 16; __VA_ARGS__; } break;                     \
    case 129: { constexpr int TPI = 8, L = 8; __VA_ARGS__; } break;                      \
    case 256: { constexpr int TPI = 8, L = 16; __VA_ARGS__; } break;                     \
    case 257: { constexpr int TPI = 4, L = 32; __VA_ARGS__; } break;                     \
    case 384: { constexpr int TPI = 16, L = 12; __VA_ARGS__; } break;                    \
    case 385: { constexpr int TPI = 8, L = 24; __VA_ARGS__; } break;                     \
    default: return cudaErrorInvalidValue;                                               \
  }

// Default variant only: kernels whose speed does not depend on the layout
// choice (single multiplications, trees, tables) instantiate just this one.
#define HG_DISPATCH_S0(S, ...)                                                           \
  switch (S) {                                                                           \
    case 64: { constexpr int TPI = 4, L = 16; __VA_ARGS__; } break;                      \
    case 128: { constexpr int TPI = 8, L = 16; __VA_ARGS__; } break;                     \
    case 192: { constexpr int TPI = 16, L = 12; __VA_ARGS__; } break;                    \
    default: return cudaErrorInvalidValue;                                               \
  }

#define HG_DISPATCH_SPV(SP, V, ...)                                                      \
  switch ((SP) * 2 + ((V) ? 1 : 0)) {                                                    \
    case 64: { constexpr int TP = 2, LP = 16; __VA_ARGS__; } break;                      \
    case 65: { constexpr int TP = 4, LP = 8; __VA_ARGS__; } break;                       \
    case 128: { constexpr int TP = 4, LP = 16; __VA_ARGS__; } break;                     \
    case 129: { constexpr int TP = 8, LP = 8; __VA_ARGS__; } break;                      \
    case 192: { constexpr int TP = 8, LP = 12; __VA_ARGS__; } break;                     \
    case 193: { constexpr int TP = 4, LP = 24; __VA_ARGS__; } break;                     \
    default: return cudaErrorInvalidValue;                                               \
  }

// Latency layout (short batches): a whole warp per instance mod n^2 and a
// half warp per CRT side mod p^2, so each dependent chain of Montgomery
// multiplications advances with 2-6 limbs per lane instead of 8-24.
#define HG_DISPATCH_SL(S, ...)                                                           \
  switch (S) {                                                                           \
    case 64: { constexpr int TPI = 32, L = 2; __VA_ARGS__; } break;                      \
    case 128: { constexpr int TPI = 32, L = 4; __VA_ARGS__; } break;                     \
    case 192: { constexpr int TPI = 32, L = 6; __VA_ARGS__; } break;                     \
    default: return cudaErrorInvalidValue;                                               \
  }

#define HG_DISPATCH_SPL(SP, ...)                                                         \
  switch (SP) {                                                                          \
    case 32: { constexpr int TP = 16, LP = 2; __VA_ARGS__; } break;                      \
    case 64: { constexpr int TP = 16, LP = 4; __VA_ARGS__; } break;                      \
    case 96: { constexpr int TP = 16, LP = 6; __VA_ARGS__; } break;                      \
    default: return cudaErrorInvalidValue;                                               \
  }

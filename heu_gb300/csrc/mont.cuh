// Distributed multi-limb Montgomery arithmetic for sm_103a.
//
// A big number of S 32-bit limbs is spread over a group of TPI consecutive
// lanes of one warp ("threads per instance"); lane t of the group holds limbs
// [t*L, t*L + L) in registers, L = S / TPI.  All groups of a warp execute the
// same instruction stream (full-warp shuffles and ballots), so every kernel
// keeps its warps converged and handles tails by computing on a dummy
// instance and skipping the store.
//
// Montgomery multiplication follows the coarsely integrated operand scanning
// (CIOS) method of Koc, Acar and Kaliski ("Analyzing and comparing Montgomery
// multiplication algorithms", IEEE Micro 1996) with R = 2^(32*S):
//   for i in 0..S-1:  T += A*b_i;  m = T_0 * n' mod 2^32;  T += m*N;  T >>= 32
// Each lane keeps its slice of T plus a small lazy carry word that belongs to
// the lowest limb of the next lane; carries between lanes are settled once at
// the end with a ballot-based carry-lookahead (generate/propagate masks added
// as integers), followed by the conditional subtraction of N.
#pragma once
#include <cstdint>

namespace hg {

constexpr uint32_t kFull = 0xffffffffu;

// ---- PTX carry-chain primitives -------------------------------------------
__device__ __forceinline__ uint32_t add_cc(uint32_t a, uint32_t b) {
  uint32_t r;
  asm volatile("add.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t addc_cc(uint32_t a, uint32_t b) {
  uint32_t r;
  asm volatile("addc.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t addc(uint32_t a, uint32_t b) {
  uint32_t r;
  asm volatile("addc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t sub_cc(uint32_t a, uint32_t b) {
  uint32_t r;
  asm volatile("sub.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t subc_cc(uint32_t a, uint32_t b) {
  uint32_t r;
  asm volatile("subc.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t subc(uint32_t a, uint32_t b) {
  uint32_t r;
  asm volatile("subc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t mad_lo_cc(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm volatile("mad.lo.cc.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t madc_lo_cc(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm volatile("madc.lo.cc.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t mad_hi_cc(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm volatile("mad.hi.cc.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t madc_hi_cc(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm volatile("madc.hi.cc.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}

// ---- group geometry --------------------------------------------------------
template <int TPI>
struct Group {
  static_assert(TPI == 2 || TPI == 4 || TPI == 8 || TPI == 16 || TPI == 32, "TPI");
  uint32_t t;     // index of this lane inside its group
  uint32_t base;  // warp lane of the group's lane 0
  __device__ __forceinline__ Group() {
    const uint32_t lane = threadIdx.x & 31u;
    t = lane & (TPI - 1);
    base = lane - t;
  }
};

// Carry-lookahead across the lanes of a group.  g: this lane's slice produced
// a carry (borrow) by itself; p: the slice would pass an incoming carry
// (borrow) through.  g and p must never both be set.  Returns the carry into
// this lane; `out` receives the carry out of the top lane.  `cin0` is a carry
// into lane 0.
template <int TPI>
__device__ __forceinline__ uint32_t lookahead(const Group<TPI>& g, bool gen, bool prop,
                                              uint32_t cin0, uint32_t& out) {
  const uint32_t G = __ballot_sync(kFull, gen);
  const uint32_t P = __ballot_sync(kFull, prop);
  const uint64_t mask = (TPI == 32) ? 0xffffffffull : ((1ull << TPI) - 1ull);
  const uint64_t Gg = (uint64_t)(G >> g.base) & mask;
  const uint64_t Pg = (uint64_t)(P >> g.base) & mask;
  const uint64_t c = ((Gg | Pg) + Gg + (uint64_t)cin0) ^ Pg;
  out = (uint32_t)(c >> TPI) & 1u;
  return (uint32_t)(c >> g.t) & 1u;
}

// ---- slices: load / store / small helpers ---------------------------------
template <int L>
__device__ __forceinline__ void load_slice(uint32_t (&x)[L], const uint32_t* __restrict__ p) {
  if constexpr (L % 4 == 0) {
    const uint4* q = reinterpret_cast<const uint4*>(p);
#pragma unroll
    for (int i = 0; i < L / 4; ++i) {
      const uint4 v = q[i];
      x[4 * i] = v.x;
      x[4 * i + 1] = v.y;
      x[4 * i + 2] = v.z;
      x[4 * i + 3] = v.w;
    }
  } else if constexpr (L % 2 == 0) {
    const uint2* q = reinterpret_cast<const uint2*>(p);
#pragma unroll
    for (int i = 0; i < L / 2; ++i) {
      const uint2 v = q[i];
      x[2 * i] = v.x;
      x[2 * i + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < L; ++i) x[i] = p[i];
  }
}

template <int L>
__device__ __forceinline__ void store_slice(uint32_t* __restrict__ p, const uint32_t (&x)[L]) {
  if constexpr (L % 4 == 0) {
    uint4* q = reinterpret_cast<uint4*>(p);
#pragma unroll
    for (int i = 0; i < L / 4; ++i) q[i] = make_uint4(x[4 * i], x[4 * i + 1], x[4 * i + 2], x[4 * i + 3]);
  } else if constexpr (L % 2 == 0) {
    uint2* q = reinterpret_cast<uint2*>(p);
#pragma unroll
    for (int i = 0; i < L / 2; ++i) q[i] = make_uint2(x[2 * i], x[2 * i + 1]);
  } else {
#pragma unroll
    for (int i = 0; i < L; ++i) p[i] = x[i];
  }
}

template <int L>
__device__ __forceinline__ void copy_slice(uint32_t (&d)[L], const uint32_t (&s)[L]) {
#pragma unroll
  for (int i = 0; i < L; ++i) d[i] = s[i];
}

template <int L>
__device__ __forceinline__ void select_slice(uint32_t (&d)[L], bool take_a, const uint32_t (&a)[L],
                                             const uint32_t (&b)[L]) {
#pragma unroll
  for (int i = 0; i < L; ++i) d[i] = take_a ? a[i] : b[i];
}

// Small value v (< 2^64) as a distributed number: limbs 0 and 1 of lane 0.
template <int TPI, int L>
__device__ __forceinline__ void set_u64(uint32_t (&x)[L], const Group<TPI>& g, uint64_t v) {
#pragma unroll
  for (int i = 0; i < L; ++i) x[i] = 0;
  if (g.t == 0) {
    x[0] = (uint32_t)v;
    if constexpr (L > 1) x[1] = (uint32_t)(v >> 32);
  }
  if constexpr (L == 1) {
    if (g.t == 1) x[0] = (uint32_t)(v >> 32);
  }
}

// ---- distributed add / sub -------------------------------------------------
// r = a + b; returns the carry out of the whole number (same in every lane).
template <int TPI, int L>
__device__ __forceinline__ uint32_t add_full(uint32_t (&r)[L], const uint32_t (&a)[L],
                                             const uint32_t (&b)[L], const Group<TPI>& g) {
  r[0] = add_cc(a[0], b[0]);
#pragma unroll
  for (int i = 1; i < L; ++i) r[i] = addc_cc(a[i], b[i]);
  const uint32_t gen = addc(0u, 0u);
  uint32_t all = r[0];
#pragma unroll
  for (int i = 1; i < L; ++i) all &= r[i];
  uint32_t out;
  const uint32_t ci = lookahead<TPI>(g, gen != 0, all == kFull, 0u, out);
  r[0] = add_cc(r[0], ci);
#pragma unroll
  for (int i = 1; i < L; ++i) r[i] = addc_cc(r[i], 0u);
  (void)addc(0u, 0u);
  return out;
}

// r = a - b; returns the borrow out of the whole number (same in every lane).
template <int TPI, int L>
__device__ __forceinline__ uint32_t sub_full(uint32_t (&r)[L], const uint32_t (&a)[L],
                                             const uint32_t (&b)[L], const Group<TPI>& g) {
  r[0] = sub_cc(a[0], b[0]);
#pragma unroll
  for (int i = 1; i < L; ++i) r[i] = subc_cc(a[i], b[i]);
  const uint32_t gen = subc(0u, 0u) & 1u;
  uint32_t any = r[0];
#pragma unroll
  for (int i = 1; i < L; ++i) any |= r[i];
  uint32_t out;
  const uint32_t bi = lookahead<TPI>(g, gen != 0, any == 0u, 0u, out);
  r[0] = sub_cc(r[0], bi);
#pragma unroll
  for (int i = 1; i < L; ++i) r[i] = subc_cc(r[i], 0u);
  (void)subc(0u, 0u);
  return out;
}

// r = (top:x) mod N for a value known to be < 2N (top is the bit above x).
template <int TPI, int L>
__device__ __forceinline__ void reduce_once(uint32_t (&r)[L], const uint32_t (&x)[L], uint32_t top,
                                            const uint32_t (&n)[L], const Group<TPI>& g) {
  uint32_t d[L];
  const uint32_t borrow = sub_full<TPI, L>(d, x, n, g);
  select_slice<L>(r, (top != 0u) || (borrow == 0u), d, x);
}

// r = a + b mod N (a, b < N)
template <int TPI, int L>
__device__ __forceinline__ void mod_add(uint32_t (&r)[L], const uint32_t (&a)[L], const uint32_t (&b)[L],
                                        const uint32_t (&n)[L], const Group<TPI>& g) {
  uint32_t s[L];
  const uint32_t c = add_full<TPI, L>(s, a, b, g);
  reduce_once<TPI, L>(r, s, c, n, g);
}

// r = a - b mod N (a, b < N)
template <int TPI, int L>
__device__ __forceinline__ void mod_sub(uint32_t (&r)[L], const uint32_t (&a)[L], const uint32_t (&b)[L],
                                        const uint32_t (&n)[L], const Group<TPI>& g) {
  uint32_t d[L], e[L];
  const uint32_t borrow = sub_full<TPI, L>(d, a, b, g);
  (void)add_full<TPI, L>(e, d, n, g);
  select_slice<L>(r, borrow != 0u, e, d);
}

// Is x == 0 (whole number)?
template <int TPI, int L>
__device__ __forceinline__ bool is_zero(const uint32_t (&x)[L], const Group<TPI>& g) {
  uint32_t any = 0;
#pragma unroll
  for (int i = 0; i < L; ++i) any |= x[i];
  const uint32_t B = __ballot_sync(kFull, any != 0u);
  const uint32_t mask = (TPI == 32) ? kFull : ((1u << TPI) - 1u);
  return ((B >> g.base) & mask) == 0u;
}

// Is x < N (whole number)?
template <int TPI, int L>
__device__ __forceinline__ bool less_than(const uint32_t (&x)[L], const uint32_t (&n)[L], const Group<TPI>& g) {
  uint32_t d[L];
  return sub_full<TPI, L>(d, x, n, g) != 0u;
}

// ---- Montgomery core -------------------------------------------------------
// T (L limbs) plus lazy carry (c0 + c1*2^32, positioned at limb L) += x * y.
// Written as plain 64-bit arithmetic: x_j*y + T_j + c never exceeds 2^64 - 1,
// and the compiler maps each step to one wide multiply-add plus the carry
// adds, which measured 20% faster on sm_103a than explicit PTX carry chains
// (mad.lo.cc / madc.hi.cc) for the same rows.
template <int L>
__device__ __forceinline__ void row_mac(uint32_t (&T)[L], uint32_t& c0, uint32_t& c1, const uint32_t (&x)[L],
                                        uint32_t y) {
  uint64_t c = 0;
#pragma unroll
  for (int j = 0; j < L; ++j) {
    const uint64_t t = (uint64_t)x[j] * y + T[j] + c;
    T[j] = (uint32_t)t;
    c = t >> 32;
  }
  const uint64_t cc = (uint64_t)c0 + c;
  c0 = (uint32_t)cc;
  c1 += (uint32_t)(cc >> 32);
}

// One CIOS reduction-and-shift step with the multiplier limb already added.
template <int TPI, int L>
__device__ __forceinline__ void shift_step(uint32_t (&T)[L], uint32_t& c0, uint32_t& c1, const Group<TPI>& g) {
  uint32_t x = __shfl_down_sync(kFull, T[0], 1, TPI);
  x = (g.t == TPI - 1) ? 0u : x;
#pragma unroll
  for (int k = 0; k < L - 1; ++k) T[k] = T[k + 1];
  T[L - 1] = add_cc(x, c0);
  c0 = addc(c1, 0u);
  c1 = 0u;
}

// Settle the lazy carries and return the bit above the top limb.
template <int TPI, int L>
__device__ __forceinline__ uint32_t settle(uint32_t (&T)[L], uint32_t c0, const Group<TPI>& g) {
  uint32_t cin = __shfl_up_sync(kFull, c0, 1, TPI);
  cin = (g.t == 0) ? 0u : cin;
  const uint32_t topc = __shfl_sync(kFull, c0, TPI - 1, TPI);
  T[0] = add_cc(T[0], cin);
#pragma unroll
  for (int i = 1; i < L; ++i) T[i] = addc_cc(T[i], 0u);
  const uint32_t gen = addc(0u, 0u);
  uint32_t all = T[0];
#pragma unroll
  for (int i = 1; i < L; ++i) all &= T[i];
  uint32_t out;
  const uint32_t ci = lookahead<TPI>(g, gen != 0, all == kFull, 0u, out);
  T[0] = add_cc(T[0], ci);
#pragma unroll
  for (int i = 1; i < L; ++i) T[i] = addc_cc(T[i], 0u);
  (void)addc(0u, 0u);
  return topc + out;
}

// r = a * b * R^-1 mod N, for a < R, b < N (result < N).  r may alias a or b.
template <int TPI, int L>
__device__ __forceinline__ void mont_mul(uint32_t (&r)[L], const uint32_t (&a)[L], const uint32_t (&b)[L],
                                         const uint32_t (&n)[L], uint32_t np, const Group<TPI>& g) {
  uint32_t T[L];
#pragma unroll
  for (int j = 0; j < L; ++j) T[j] = 0u;
  uint32_t c0 = 0u, c1 = 0u;
#pragma unroll 1
  for (int owner = 0; owner < TPI; ++owner) {
#pragma unroll
    for (int j = 0; j < L; ++j) {
      const uint32_t bi = __shfl_sync(kFull, b[j], owner, TPI);
      uint32_t m = (T[0] + a[0] * bi) * np;
      m = __shfl_sync(kFull, m, 0, TPI);
      row_mac<L>(T, c0, c1, a, bi);
      row_mac<L>(T, c0, c1, n, m);
      shift_step<TPI, L>(T, c0, c1, g);
    }
  }
  const uint32_t top = settle<TPI, L>(T, c0, g);
  reduce_once<TPI, L>(r, T, top, n, g);
}

// r = a * R^-1 mod N (Montgomery reduction of a single-width a < R).
template <int TPI, int L>
__device__ __forceinline__ void mont_redc(uint32_t (&r)[L], const uint32_t (&a)[L], const uint32_t (&n)[L],
                                          uint32_t np, const Group<TPI>& g) {
  uint32_t T[L];
  copy_slice<L>(T, a);
  uint32_t c0 = 0u, c1 = 0u;
#pragma unroll 1
  for (int owner = 0; owner < TPI; ++owner) {
#pragma unroll
    for (int j = 0; j < L; ++j) {
      uint32_t m = T[0] * np;
      m = __shfl_sync(kFull, m, 0, TPI);
      row_mac<L>(T, c0, c1, n, m);
      shift_step<TPI, L>(T, c0, c1, g);
    }
  }
  const uint32_t top = settle<TPI, L>(T, c0, g);
  reduce_once<TPI, L>(r, T, top, n, g);
}

// r = (hi*R + lo) * R^-1 mod N for a double-width input (hi:lo) < N*R.
template <int TPI, int L>
__device__ __forceinline__ void mont_redc_wide(uint32_t (&r)[L], const uint32_t (&lo)[L], const uint32_t (&hi)[L],
                                               const uint32_t (&n)[L], uint32_t np, const Group<TPI>& g) {
  uint32_t T[L];
  copy_slice<L>(T, lo);
  uint32_t c0 = 0u, c1 = 0u;
#pragma unroll 1
  for (int owner = 0; owner < TPI; ++owner) {
#pragma unroll
    for (int j = 0; j < L; ++j) {
      uint32_t m = T[0] * np;
      m = __shfl_sync(kFull, m, 0, TPI);
      row_mac<L>(T, c0, c1, n, m);
      shift_step<TPI, L>(T, c0, c1, g);
    }
  }
  const uint32_t top = settle<TPI, L>(T, c0, g);  // T <= N here, top == 0
  uint32_t s[L];
  const uint32_t c = add_full<TPI, L>(s, T, hi, g);
  reduce_once<TPI, L>(r, s, c + top, n, g);
}

}  // namespace hg

// Host-side arbitrary-precision unsigned integers for key generation and key
// precompute (nothing on the per-ciphertext path).  Portable C++17: 32-bit
// limbs with 64-bit intermediates, no compiler intrinsics, so x86-64 and
// aarch64 hosts produce identical keys from the same seed.
//
// Also holds the seeded stream used when a key is generated from a seed:
// xoshiro256** (Blackman & Vigna 2018) seeded through SplitMix64.
#pragma once
#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace hg {

class BN {
 public:
  std::vector<uint32_t> d;  // little-endian limbs, no leading zero limbs

  BN() = default;
  explicit BN(uint64_t v) {
    if (v) d.push_back((uint32_t)v);
    if (v >> 32) d.push_back((uint32_t)(v >> 32));
  }
  static BN from_limbs(const uint32_t* p, size_t n) {
    BN r;
    r.d.assign(p, p + n);
    r.trim();
    return r;
  }
  void to_limbs(uint32_t* p, size_t n) const {
    if (d.size() > n) throw std::runtime_error("BN does not fit in limbs");
    for (size_t i = 0; i < n; ++i) p[i] = i < d.size() ? d[i] : 0u;
  }
  std::vector<uint32_t> limbs(size_t n) const {
    std::vector<uint32_t> v(n);
    to_limbs(v.data(), n);
    return v;
  }
  void trim() {
    while (!d.empty() && d.back() == 0) d.pop_back();
  }
  bool is_zero() const { return d.empty(); }
  bool is_odd() const { return !d.empty() && (d[0] & 1u); }
  size_t bitlen() const {
    if (d.empty()) return 0;
    uint32_t top = d.back();
    size_t b = 0;
    while (top) {
      ++b;
      top >>= 1;
    }
    return 32 * (d.size() - 1) + b;
  }
  bool bit(size_t i) const {
    const size_t w = i / 32;
    return w < d.size() && ((d[w] >> (i % 32)) & 1u);
  }
  uint64_t low64() const {
    uint64_t v = d.empty() ? 0 : d[0];
    if (d.size() > 1) v |= (uint64_t)d[1] << 32;
    return v;
  }

  static int cmp(const BN& a, const BN& b) {
    if (a.d.size() != b.d.size()) return a.d.size() < b.d.size() ? -1 : 1;
    for (size_t i = a.d.size(); i-- > 0;) {
      if (a.d[i] != b.d[i]) return a.d[i] < b.d[i] ? -1 : 1;
    }
    return 0;
  }
  friend bool operator==(const BN& a, const BN& b) { return cmp(a, b) == 0; }
  friend bool operator!=(const BN& a, const BN& b) { return cmp(a, b) != 0; }
  friend bool operator<(const BN& a, const BN& b) { return cmp(a, b) < 0; }
  friend bool operator<=(const BN& a, const BN& b) { return cmp(a, b) <= 0; }
  friend bool operator>(const BN& a, const BN& b) { return cmp(a, b) > 0; }
  friend bool operator>=(const BN& a, const BN& b) { return cmp(a, b) >= 0; }

  friend BN operator+(const BN& a, const BN& b) {
    BN r;
    const size_t n = std::max(a.d.size(), b.d.size());
    r.d.resize(n + 1);
    uint64_t c = 0;
    for (size_t i = 0; i < n; ++i) {
      c += (uint64_t)(i < a.d.size() ? a.d[i] : 0) + (i < b.d.size() ? b.d[i] : 0);
      r.d[i] = (uint32_t)c;
      c >>= 32;
    }
    r.d[n] = (uint32_t)c;
    r.trim();
    return r;
  }
  // a - b, requires a >= b
  friend BN operator-(const BN& a, const BN& b) {
    if (a < b) throw std::runtime_error("BN subtraction underflow");
    BN r;
    r.d.resize(a.d.size());
    int64_t br = 0;
    for (size_t i = 0; i < a.d.size(); ++i) {
      int64_t v = (int64_t)a.d[i] - (i < b.d.size() ? b.d[i] : 0) - br;
      br = v < 0;
      r.d[i] = (uint32_t)(v + (br << 32));
    }
    r.trim();
    return r;
  }
  friend BN operator*(const BN& a, const BN& b) {
    BN r;
    if (a.is_zero() || b.is_zero()) return r;
    r.d.assign(a.d.size() + b.d.size(), 0);
    for (size_t i = 0; i < a.d.size(); ++i) {
      uint64_t c = 0;
      for (size_t j = 0; j < b.d.size(); ++j) {
        c += (uint64_t)a.d[i] * b.d[j] + r.d[i + j];
        r.d[i + j] = (uint32_t)c;
        c >>= 32;
      }
      r.d[i + b.d.size()] = (uint32_t)c;
    }
    r.trim();
    return r;
  }
  BN shl(size_t k) const {
    if (is_zero()) return *this;
    BN r;
    const size_t w = k / 32, s = k % 32;
    r.d.assign(d.size() + w + 1, 0);
    for (size_t i = 0; i < d.size(); ++i) {
      r.d[i + w] |= d[i] << s;
      if (s) r.d[i + w + 1] |= d[i] >> (32 - s);
    }
    r.trim();
    return r;
  }
  BN shr(size_t k) const {
    const size_t w = k / 32, s = k % 32;
    if (w >= d.size()) return BN();
    BN r;
    r.d.assign(d.size() - w, 0);
    for (size_t i = 0; i < r.d.size(); ++i) {
      uint64_t v = d[i + w];
      if (i + w + 1 < d.size()) v |= (uint64_t)d[i + w + 1] << 32;
      r.d[i] = (uint32_t)(v >> s);
    }
    r.trim();
    return r;
  }
  // low k bits
  BN mask_bits(size_t k) const {
    BN r = *this;
    const size_t w = (k + 31) / 32;
    if (r.d.size() > w) r.d.resize(w);
    if (k % 32 && r.d.size() == w) r.d[w - 1] &= (1u << (k % 32)) - 1u;
    r.trim();
    return r;
  }

  // Knuth algorithm D (TAOCP vol. 2, 4.3.1): q = a / b, r = a % b.
  static void divmod(const BN& a, const BN& b, BN* q, BN* r) {
    if (b.is_zero()) throw std::runtime_error("BN division by zero");
    if (a < b) {
      if (q) *q = BN();
      if (r) *r = a;
      return;
    }
    if (b.d.size() == 1) {
      BN qq;
      qq.d.assign(a.d.size(), 0);
      uint64_t rem = 0;
      for (size_t i = a.d.size(); i-- > 0;) {
        const uint64_t cur = (rem << 32) | a.d[i];
        qq.d[i] = (uint32_t)(cur / b.d[0]);
        rem = cur % b.d[0];
      }
      qq.trim();
      if (q) *q = qq;
      if (r) *r = BN(rem);
      return;
    }
    // normalise
    size_t s = 0;
    uint32_t top = b.d.back();
    while (!(top & 0x80000000u)) {
      top <<= 1;
      ++s;
    }
    const BN bn = b.shl(s);
    BN an = a.shl(s);
    const size_t n = bn.d.size();
    if (an.d.size() == a.d.size()) an.d.push_back(0);
    if (an.d.size() < a.d.size() + 1) an.d.resize(a.d.size() + 1, 0);
    const size_t m = an.d.size() - n;
    BN qq;
    qq.d.assign(m, 0);
    const uint64_t btop = bn.d[n - 1], bnext = bn.d[n - 2];
    for (size_t j = m; j-- > 0;) {
      const uint64_t num = ((uint64_t)an.d[j + n] << 32) | an.d[j + n - 1];
      uint64_t qhat = num / btop;
      uint64_t rhat = num % btop;
      while (qhat > 0xffffffffull || qhat * bnext > ((rhat << 32) | an.d[j + n - 2])) {
        --qhat;
        rhat += btop;
        if (rhat > 0xffffffffull) break;
      }
      // multiply-subtract
      int64_t borrow = 0;
      uint64_t carry = 0;
      for (size_t i = 0; i < n; ++i) {
        const uint64_t p = qhat * bn.d[i] + carry;
        carry = p >> 32;
        const int64_t t = (int64_t)an.d[i + j] - (int64_t)(uint32_t)p - borrow;
        an.d[i + j] = (uint32_t)t;
        borrow = t < 0 ? 1 : 0;
      }
      const int64_t t = (int64_t)an.d[j + n] - (int64_t)carry - borrow;
      an.d[j + n] = (uint32_t)t;
      if (t < 0) {
        --qhat;
        uint64_t c = 0;
        for (size_t i = 0; i < n; ++i) {
          c += (uint64_t)an.d[i + j] + bn.d[i];
          an.d[i + j] = (uint32_t)c;
          c >>= 32;
        }
        an.d[j + n] += (uint32_t)c;
      }
      qq.d[j] = (uint32_t)qhat;
    }
    qq.trim();
    if (q) *q = qq;
    if (r) {
      an.d.resize(n);
      an.trim();
      *r = an.shr(s);
    }
  }
  friend BN operator%(const BN& a, const BN& b) {
    BN r;
    divmod(a, b, nullptr, &r);
    return r;
  }
  friend BN operator/(const BN& a, const BN& b) {
    BN q;
    divmod(a, b, &q, nullptr);
    return q;
  }

  static BN gcd(BN a, BN b) {
    while (!b.is_zero()) {
      BN r = a % b;
      a = std::move(b);
      b = std::move(r);
    }
    return a;
  }

  // a^-1 mod m (throws if not invertible).  Extended Euclid with the
  // Bezout coefficient of a tracked modulo m.
  static BN invmod(const BN& a_in, const BN& m) {
    BN a = a_in % m;
    BN r0 = m, r1 = a;
    BN t0, t1(1);  // t coefficients mod m
    while (!r1.is_zero()) {
      BN q, r2;
      divmod(r0, r1, &q, &r2);
      // t2 = t0 - q*t1 mod m
      const BN qt = (q * t1) % m;
      BN t2 = (t0 >= qt) ? (t0 - qt) : (m - (qt - t0));
      r0 = std::move(r1);
      r1 = std::move(r2);
      t0 = std::move(t1);
      t1 = std::move(t2);
    }
    if (r0 != BN(1)) throw std::runtime_error("BN invmod: not invertible");
    return t0 % m;
  }

  static BN mulmod(const BN& a, const BN& b, const BN& m) { return (a * b) % m; }

  // a^e mod m by left-to-right binary exponentiation (setup only).
  static BN powmod(const BN& a, const BN& e, const BN& m) {
    BN r(1);
    r = r % m;
    const BN base = a % m;
    for (size_t i = e.bitlen(); i-- > 0;) {
      r = mulmod(r, r, m);
      if (e.bit(i)) r = mulmod(r, base, m);
    }
    return r;
  }
};


// Montgomery form of the inverse of a Montgomery residue, for the root of
// the batch-inversion trees: given xr = X*R mod N (N odd, R = 2^(32*S)),
// returns X^-1 * R mod N as S 32-bit limbs, or false if gcd(X, N) != 1.
// Kaliski's almost Montgomery inverse ("The Montgomery inverse and its
// applications", IEEE Trans. Computers 1995) computes w = xr^-1 * 2^k with
// shifts and adds only; then X^-1 * R = w * 2^(2*32*S - k) mod N.  Runs of
// zero bits are shifted out at once and the working lengths shrink / grow
// with the operands.
inline bool mont_root_inverse(const uint32_t* xr, const BN& N, size_t S, uint32_t* out) {
  const size_t n = (S + 1) / 2 + 1;  // 64-bit words with one word of slack
  std::vector<uint64_t> u(n, 0), v(n, 0), r(n + 1, 0), s(n + 1, 0);
  for (size_t i = 0; i < S; ++i) v[i / 2] |= (uint64_t)xr[i] << (32 * (i % 2));
  for (size_t i = 0; i < N.d.size(); ++i) u[i / 2] |= (uint64_t)N.d[i] << (32 * (i % 2));
  auto len_of = [](const std::vector<uint64_t>& a, size_t hint) {
    while (hint > 0 && a[hint - 1] == 0) --hint;
    return hint;
  };
  auto ctz64 = [](uint64_t x) {
    int c = 0;
    while (!(x & 1)) {
      x >>= 1;
      ++c;
    }
    return c;
  };
  // a >>= t (t < 64) over len words
  auto shr = [](std::vector<uint64_t>& a, size_t len, int t) {
    if (t == 0) return;
    for (size_t i = 0; i + 1 < len; ++i) a[i] = (a[i] >> t) | (a[i + 1] << (64 - t));
    a[len - 1] >>= t;
  };
  // a <<= t (t < 64) over len words (len includes room for the carry-out)
  auto shl = [](std::vector<uint64_t>& a, size_t len, int t) {
    if (t == 0) return;
    for (size_t i = len - 1; i > 0; --i) a[i] = (a[i] << t) | (a[i - 1] >> (64 - t));
    a[0] <<= t;
  };
  auto cmp = [](const std::vector<uint64_t>& a, const std::vector<uint64_t>& b, size_t len) {
    for (size_t i = len; i-- > 0;)
      if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
    return 0;
  };
  auto sub = [](std::vector<uint64_t>& a, const std::vector<uint64_t>& b, size_t len) {
    uint64_t br = 0;
    for (size_t i = 0; i < len; ++i) {
      const uint64_t ai = a[i], bi = b[i];
      a[i] = ai - bi - br;
      br = (ai < bi) | ((ai == bi) & br);
    }
  };
  auto add = [](std::vector<uint64_t>& a, const std::vector<uint64_t>& b, size_t len) {
    uint64_t c = 0;
    for (size_t i = 0; i < len; ++i) {
      const uint64_t t = a[i] + c;
      const uint64_t c1 = t < c;
      a[i] = t + b[i];
      c = c1 | (a[i] < t);
    }
  };
  s[0] = 1;
  size_t luv = n, lrs = 1;
  size_t k = 0;
  luv = std::max(len_of(u, n), len_of(v, n));
  if (luv == 0) return false;
  while (true) {
    const size_t lv = len_of(v, luv);
    if (lv == 0) break;
    if (!(u[0] & 1)) {
      int t = 0;
      while (u[0] == 0) {  // whole zero words
        for (size_t i = 0; i + 1 < luv; ++i) u[i] = u[i + 1];
        u[luv - 1] = 0;
        for (size_t i = lrs + 1; i-- > 1;) s[i] = s[i - 1];
        s[0] = 0;
        lrs = std::min(lrs + 1, n);
        k += 64;
      }
      t = ctz64(u[0]);
      shr(u, luv, t);
      lrs = std::min(lrs + 1, n);
      shl(s, lrs + 1, t);
      k += (size_t)t;
    } else if (!(v[0] & 1)) {
      int t = 0;
      while (v[0] == 0) {
        for (size_t i = 0; i + 1 < luv; ++i) v[i] = v[i + 1];
        v[luv - 1] = 0;
        for (size_t i = lrs + 1; i-- > 1;) r[i] = r[i - 1];
        r[0] = 0;
        lrs = std::min(lrs + 1, n);
        k += 64;
      }
      t = ctz64(v[0]);
      shr(v, luv, t);
      lrs = std::min(lrs + 1, n);
      shl(r, lrs + 1, t);
      k += (size_t)t;
    } else if (cmp(u, v, luv) > 0) {
      sub(u, v, luv);
      add(r, s, lrs + 1);
    } else {
      sub(v, u, luv);
      add(s, r, lrs + 1);
    }
    luv = std::max<size_t>(1, std::max(len_of(u, luv), len_of(v, luv)));
    lrs = std::max(len_of(r, lrs + 1), len_of(s, lrs + 1));
  }
  // gcd is u; invertible only if u == 1
  if (!(u[0] == 1 && len_of(u, luv) == 1)) return false;
  // w = N - (r mod N)
  std::vector<uint32_t> rw(2 * (n + 1));
  for (size_t i = 0; i < n + 1; ++i) {
    rw[2 * i] = (uint32_t)r[i];
    rw[2 * i + 1] = (uint32_t)(r[i] >> 32);
  }
  BN rb = BN::from_limbs(rw.data(), rw.size()) % N;
  const BN w = rb.is_zero() ? BN() : N - rb;
  const size_t two_bits = 2 * 32 * S;
  if (k > two_bits) return false;
  const BN z = w.shl(two_bits - k) % N;
  z.to_limbs(out, S);
  return true;
}

// Montgomery context over an odd modulus with 32-bit limbs, used by the
// Miller-Rabin test during key generation (many modexps).
class HostMont {
 public:
  explicit HostMont(const BN& m) : m_(m), s_(m.d.size()) {
    // np = -m^-1 mod 2^32 by Newton iteration
    uint32_t inv = 1;
    for (int i = 0; i < 5; ++i) inv *= 2u - m.d[0] * inv;
    np_ = 0u - inv;
    const BN R = BN(1).shl(32 * s_);
    r1_ = R % m;
    r2_ = (r1_ * r1_) % m;
  }
  std::vector<uint32_t> to(const BN& a) const { return mul(pad(a % m_), pad(r2_)); }
  BN from(const std::vector<uint32_t>& a) const {
    std::vector<uint32_t> one(s_, 0);
    one[0] = 1;
    return BN::from_limbs(mul(a, one).data(), s_);
  }
  std::vector<uint32_t> one() const { return pad(r1_); }
  std::vector<uint32_t> mul(const std::vector<uint32_t>& a, const std::vector<uint32_t>& b) const {
    std::vector<uint32_t> t(s_ + 2, 0);
    for (size_t i = 0; i < s_; ++i) {
      uint64_t c = 0;
      for (size_t j = 0; j < s_; ++j) {
        c += (uint64_t)a[j] * b[i] + t[j];
        t[j] = (uint32_t)c;
        c >>= 32;
      }
      c += t[s_];
      t[s_] = (uint32_t)c;
      t[s_ + 1] = (uint32_t)(c >> 32);
      const uint32_t mq = t[0] * np_;
      c = (uint64_t)mq * m_.d[0] + t[0];
      c >>= 32;
      for (size_t j = 1; j < s_; ++j) {
        c += (uint64_t)mq * m_.d[j] + t[j];
        t[j - 1] = (uint32_t)c;
        c >>= 32;
      }
      c += t[s_];
      t[s_ - 1] = (uint32_t)c;
      t[s_] = t[s_ + 1] + (uint32_t)(c >> 32);
    }
    // conditional subtract
    bool ge = t[s_] != 0;
    if (!ge) {
      ge = true;
      for (size_t i = s_; i-- > 0;) {
        if (t[i] != m_.d[i]) {
          ge = t[i] > m_.d[i];
          break;
        }
      }
    }
    std::vector<uint32_t> r(t.begin(), t.begin() + s_);
    if (ge) {
      int64_t br = 0;
      for (size_t i = 0; i < s_; ++i) {
        int64_t v = (int64_t)r[i] - m_.d[i] - br;
        br = v < 0;
        r[i] = (uint32_t)(v + (br << 32));
      }
    }
    return r;
  }
  BN pow(const BN& a, const BN& e) const {
    std::vector<uint32_t> base = to(a), r = one();
    for (size_t i = e.bitlen(); i-- > 0;) {
      r = mul(r, r);
      if (e.bit(i)) r = mul(r, base);
    }
    return from(r);
  }
  std::vector<uint32_t> pad(const BN& a) const { return a.limbs(s_); }

 private:
  BN m_;
  size_t s_;
  uint32_t np_;
  BN r1_, r2_;
};

// SplitMix64-seeded xoshiro256**.
class Xoshiro {
 public:
  explicit Xoshiro(uint64_t seed) {
    uint64_t st = seed;
    for (int i = 0; i < 4; ++i) {
      st += 0x9E3779B97F4A7C15ull;
      uint64_t z = st;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      s_[i] = z ^ (z >> 31);
    }
  }
  uint64_t next() {
    const uint64_t result = rotl(s_[1] * 5, 7) * 9;
    const uint64_t t = s_[1] << 17;
    s_[2] ^= s_[0];
    s_[3] ^= s_[1];
    s_[1] ^= s_[2];
    s_[0] ^= s_[3];
    s_[2] ^= t;
    s_[3] = rotl(s_[3], 45);
    return result;
  }
  // uniform in [0, 2^k): ceil(k/64) outputs, first = least significant
  BN randbits(size_t k) {
    std::vector<uint32_t> w;
    const size_t words = (k + 63) / 64;
    for (size_t i = 0; i < words; ++i) {
      const uint64_t v = next();
      w.push_back((uint32_t)v);
      w.push_back((uint32_t)(v >> 32));
    }
    return BN::from_limbs(w.data(), w.size()).mask_bits(k);
  }
  BN below(const BN& n) {
    const size_t k = n.bitlen();
    while (true) {
      BN v = randbits(k);
      if (v < n) return v;
    }
  }

 private:
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t s_[4];
};

}  // namespace hg

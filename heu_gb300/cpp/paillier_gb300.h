// C++ schema adapter: HEU's vectorized (span-of-pointers) SPI over the
// engine's C-ABI (include/heu_gb300.h).
//
// Mirrors the classes, method names, argument meaning and error behaviour of
// heu/library/algorithms/paillier_zahlen (keys, Ciphertext) and of the
// vectorized SPI templates heu/library/algorithms/clean_template/
// vector_encryptor.h:24-33, vector_decryptor.h:25-31, vector_evaluator.h:24-66,
// so that a HEU build registers it as a new schema at the five points of
// heu/library/phe/base/schema.h:31-100 and schema.cc:35-64.  Outside
// HEU, `BigInt` and `Span` below are small stand-ins for yacl::math::BigInt
// and absl::Span<T* const>; inside HEU they are replaced by those types.
//
// Ciphertext::c_ holds the Montgomery form c*R mod n^2 with R = 2^(32*S), the
// representation paillier_z keeps (encryptor.cc:46-49).  Every ciphertext
// operation runs on the GPU; only plaintext-plaintext operations and key
// bookkeeping run on the host.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/heu_gb300.h"
#include "../csrc/host_bn.hpp"

namespace heu::lib::algorithms {

// absl::Span<T* const> stand-in: a view of `size` pointers.
template <typename P>
class SpanOf {
 public:
  SpanOf() = default;
  SpanOf(P* data, size_t size) : data_(data), size_(size) {}
  // implicit from a vector of pointers, as absl::Span; the view does not
  // extend the vector's lifetime
  template <typename V>
  SpanOf(const V& v) : data_(v.data()), size_(v.size()) {}  // NOLINT
  size_t size() const { return size_; }
  bool empty() const { return size_ == 0; }
  P& operator[](size_t i) const { return data_[i]; }
  P* begin() const { return data_; }
  P* end() const { return data_ + size_; }

 private:
  P* data_ = nullptr;
  size_t size_ = 0;
};

template <typename T>
using Span = SpanOf<T* const>;
template <typename T>
using ConstSpan = SpanOf<const T* const>;

}  // namespace heu::lib::algorithms

namespace heu::lib::algorithms::paillier_gb300 {

// ---------------------------------------------------------------------------
// BigInt: signed arbitrary-precision integer (the subset the SPI uses)
// ---------------------------------------------------------------------------
class BigInt {
 public:
  BigInt() = default;
  BigInt(int64_t v) : neg_(v < 0), mag_(v < 0 ? (uint64_t)0 - (uint64_t)v : (uint64_t)v) {}  // NOLINT
  static BigInt FromMag(hg::BN mag, bool neg) {
    BigInt r;
    r.mag_ = std::move(mag);
    r.neg_ = neg && !r.mag_.is_zero();
    return r;
  }
  static BigInt FromHex(const std::string& hex) {
    size_t i = 0;
    bool neg = false;
    if (!hex.empty() && hex[0] == '-') {
      neg = true;
      i = 1;
    }
    hg::BN m;
    for (; i < hex.size(); ++i) {
      const char c = hex[i];
      const uint32_t d = (c >= '0' && c <= '9') ? c - '0' : (c >= 'a' && c <= 'f') ? c - 'a' + 10 : c - 'A' + 10;
      m = m.shl(4) + hg::BN(d);
    }
    return FromMag(m, neg);
  }
  bool IsNegative() const { return neg_; }
  bool IsZero() const { return mag_.is_zero(); }
  size_t BitCount() const { return mag_.bitlen(); }
  const hg::BN& Mag() const { return mag_; }
  int CompareAbs(const BigInt& o) const { return hg::BN::cmp(mag_, o.mag_); }
  template <typename T>
  T Get() const;
  std::string ToHexString() const {
    static const char* dig = "0123456789ABCDEF";
    std::string s;
    if (mag_.is_zero()) return "0";
    for (size_t i = mag_.d.size(); i-- > 0;)
      for (int b = 28; b >= 0; b -= 4) s.push_back(dig[(mag_.d[i] >> b) & 0xf]);
    s.erase(0, s.find_first_not_of('0'));
    return (neg_ ? "-" : "") + s;
  }
  BigInt operator-() const { return FromMag(mag_, !neg_); }
  friend BigInt operator+(const BigInt& a, const BigInt& b) {
    if (a.neg_ == b.neg_) return FromMag(a.mag_ + b.mag_, a.neg_);
    if (hg::BN::cmp(a.mag_, b.mag_) >= 0) return FromMag(a.mag_ - b.mag_, a.neg_);
    return FromMag(b.mag_ - a.mag_, b.neg_);
  }
  friend BigInt operator-(const BigInt& a, const BigInt& b) { return a + (-b); }
  friend BigInt operator*(const BigInt& a, const BigInt& b) { return FromMag(a.mag_ * b.mag_, a.neg_ != b.neg_); }
  friend bool operator==(const BigInt& a, const BigInt& b) { return a.neg_ == b.neg_ && a.mag_ == b.mag_; }
  friend bool operator!=(const BigInt& a, const BigInt& b) { return !(a == b); }

 private:
  bool neg_ = false;
  hg::BN mag_;
};

template <>
inline int64_t BigInt::Get<int64_t>() const {
  if (mag_.bitlen() > 64) throw std::out_of_range("BigInt does not fit int64");
  const uint64_t m = mag_.low64();
  return neg_ ? (int64_t)((uint64_t)0 - m) : (int64_t)m;
}

using Plaintext = BigInt;

class Ciphertext {
 public:
  Ciphertext() = default;
  explicit Ciphertext(BigInt c) : c_(std::move(c)) {}
  std::string ToString() const { return c_.ToHexString(); }
  bool operator==(const Ciphertext& o) const { return c_ == o.c_; }
  bool operator!=(const Ciphertext& o) const { return !(*this == o); }
  BigInt c_;
};

// ---------------------------------------------------------------------------
// engine plumbing: one context per process, keys loaded once per modulus
// ---------------------------------------------------------------------------
namespace detail {

inline void Check(int rc) {
  if (rc != HG_OK) throw std::runtime_error(std::string("GB300 Paillier: ") + hg_last_error());
}

struct Engine {
  hg_ctx* ctx = nullptr;
  std::mutex mu;
  std::map<std::string, int> keys;  // "n-hex|secret" -> key id
  size_t table_window = 12;
  std::unique_ptr<hg::Xoshiro> test_stream;  // deterministic r for tests
  std::mt19937_64 rng{std::random_device{}()};
  static Engine& Get() {
    static Engine e;
    std::lock_guard<std::mutex> lk(e.mu);
    if (!e.ctx) Check(hg_ctx_create(0, &e.ctx));
    return e;
  }
};

inline void ToLimbs(const hg::BN& v, uint32_t* out, size_t n) { v.to_limbs(out, n); }
inline hg::BN FromLimbs(const uint32_t* p, size_t n) { return hg::BN::from_limbs(p, n); }

}  // namespace detail

// The density parameter of the fixed-base table (public_key.h:24-26).
inline void SetCacheTableDensity(size_t density) {
  if (density == 0) throw std::invalid_argument("density must > 0");
  auto& e = detail::Engine::Get();
  std::lock_guard<std::mutex> lk(e.mu);
  e.table_window = density;
}

// Encryption randomness from a seeded stream instead of the OS generator (tests).
inline void SetRandomStreamForTesting(uint64_t seed) {
  auto& e = detail::Engine::Get();
  std::lock_guard<std::mutex> lk(e.mu);
  e.test_stream = std::make_unique<hg::Xoshiro>(seed);
}

class SecretKey;

class PublicKey {
 public:
  BigInt n_;         // public modulus n = p * q
  BigInt n_square_;  // n_ * n_
  BigInt n_half_;    // n_ / 2
  BigInt h_s_;       // h^n mod n^2
  size_t key_size_ = 0;

  void Init() {
    n_square_ = n_ * n_;
    n_half_ = BigInt::FromMag(n_.Mag().shr(1), false);
    key_size_ = n_.BitCount();
  }
  const BigInt& PlaintextBound() const& { return n_half_; }
  bool operator==(const PublicKey& o) const { return n_ == o.n_ && h_s_ == o.h_s_; }
  bool operator!=(const PublicKey& o) const { return !(*this == o); }
  std::string ToString() const { return "GB300 Z-paillier PK: n=" + n_.ToHexString(); }
  size_t Limbs() const { return (key_size_ + 31) / 32 * 2; }  // 32-bit limbs of n^2
  size_t KeyBits() const { return Limbs() * 16; }

  // Montgomery radix 2^bits of the yacl BigInt backend the HEU build uses
  // for Ciphertext::c_ (0 = this engine's 2^(32 * Limbs()), which is the
  // radix of the 64-bit-limb OpenSSL and GMP backends; libtommath's 60-bit
  // digits give 2^(60 * ceil(bits(n^2) / 60))).  Ciphertexts cross the
  // adapter in that radix and are converted on the GPU (hg_convert_radix).
  void SetBackendRadixBits(size_t bits) { radix_bits_ = bits; }
  size_t BackendRadixBits() const { return radix_bits_ ? radix_bits_ : 32 * Limbs(); }

 private:
  size_t radix_bits_ = 0;
};

class SecretKey {
 public:
  BigInt lambda_, mu_, p_, q_;
  void Init() {}
  bool operator==(const SecretKey& o) const { return p_ == o.p_ && q_ == o.q_; }
  std::string ToString() const { return "GB300 Z-paillier SK"; }
};

namespace detail {

inline int KeyId(const PublicKey& pk, const SecretKey* sk) {
  auto& e = Engine::Get();
  const std::string tag = pk.n_.ToHexString() + (sk ? "|s" : "|p");
  std::lock_guard<std::mutex> lk(e.mu);
  auto it = e.keys.find(tag);
  if (it != e.keys.end()) return it->second;
  const size_t S = pk.Limbs(), bits = pk.KeyBits();
  std::vector<uint32_t> n(S / 2), hs(S), p(S / 4), q(S / 4);
  ToLimbs(pk.n_.Mag(), n.data(), S / 2);
  ToLimbs(pk.h_s_.Mag(), hs.data(), S);
  if (sk) {
    ToLimbs(sk->p_.Mag(), p.data(), S / 4);
    ToLimbs(sk->q_.Mag(), q.data(), S / 4);
  }
  int id = 0;
  Check(hg_key_load(e.ctx, (uint32_t)bits, n.data(), hs.data(), sk ? p.data() : nullptr, sk ? q.data() : nullptr,
                    (int)e.table_window, &id));
  e.keys[tag] = id;
  return id;
}

// r values for `count` encryptions (RandomExactBits(k/2), encryptor.cc:27)
inline std::vector<uint32_t> DrawR(const PublicKey& pk, size_t count) {
  auto& e = Engine::Get();
  const size_t rl = pk.KeyBits() / 64, rbits = pk.key_size_ / 2;
  std::vector<uint32_t> r(count * rl, 0);
  std::lock_guard<std::mutex> lk(e.mu);
  for (size_t i = 0; i < count; ++i) {
    hg::BN v;
    if (e.test_stream) {
      v = e.test_stream->randbits(rbits);
    } else {
      std::vector<uint32_t> w(rl);
      for (auto& x : w) x = (uint32_t)e.rng();
      v = hg::BN::from_limbs(w.data(), rl).mask_bits(rbits);
    }
    v.to_limbs(&r[i * rl], rl);
  }
  return r;
}

// Ciphertext limbs between the backend's radix and the engine's.
inline void ConvertRadix(const PublicKey& pk, std::vector<uint32_t>* v, bool to_backend) {
  const size_t S = pk.Limbs();
  if (pk.BackendRadixBits() == 32 * S || v->empty()) return;
  Check(hg_convert_radix(Engine::Get().ctx, KeyId(pk, nullptr), v->data(), v->data(), v->size() / S,
                         (uint32_t)pk.BackendRadixBits(), to_backend ? 1 : 0));
}

inline std::vector<uint32_t> CtLimbs(const PublicKey& pk, ConstSpan<Ciphertext> cts) {
  const size_t S = pk.Limbs();
  std::vector<uint32_t> v(cts.size() * S);
  for (size_t i = 0; i < cts.size(); ++i) {
    if (cts[i]->c_.IsNegative()) throw std::invalid_argument("Evaluator: Invalid ciphertext");
    ToLimbs(cts[i]->c_.Mag(), &v[i * S], S);
  }
  ConvertRadix(pk, &v, false);
  return v;
}

inline std::vector<Ciphertext> ToCts(const PublicKey& pk, std::vector<uint32_t> v) {
  const size_t S = pk.Limbs();
  ConvertRadix(pk, &v, true);
  std::vector<Ciphertext> out(v.size() / S);
  for (size_t i = 0; i < out.size(); ++i) out[i].c_ = BigInt::FromMag(FromLimbs(&v[i * S], S), false);
  return out;
}

inline bool AllInt64(ConstSpan<Plaintext> pts) {
  for (auto* p : pts)
    if (p->BitCount() > 63) return false;
  return true;
}

// |m| <= n/2 (encryptor.cc:38-40), checked before any r is drawn
inline void CheckPlaintexts(const PublicKey& pk, ConstSpan<Plaintext> pts) {
  for (auto* p : pts)
    if (p->CompareAbs(pk.PlaintextBound()) > 0) throw std::invalid_argument("message number out of range");
}

// Encrypt plaintexts with the given r limbs (int64 fast path or full range).
inline std::vector<uint32_t> EncryptLimbs(const PublicKey& pk, ConstSpan<Plaintext> pts, const uint32_t* r) {
  const size_t n = pts.size(), S = pk.Limbs();
  CheckPlaintexts(pk, pts);
  std::vector<uint32_t> ct(n * S);
  hg_ctx* ctx = Engine::Get().ctx;
  const int id = KeyId(pk, nullptr);
  if (AllInt64(pts)) {
    std::vector<int64_t> m(n);
    for (size_t i = 0; i < n; ++i) m[i] = pts[i]->Get<int64_t>();
    Check(hg_encrypt(ctx, id, m.data(), r, ct.data(), n));
  } else {
    std::vector<uint32_t> mag(n * (S / 2));
    std::vector<uint8_t> neg(n);
    for (size_t i = 0; i < n; ++i) {
      ToLimbs(pts[i]->Mag(), &mag[i * (S / 2)], S / 2);
      neg[i] = pts[i]->IsNegative() ? 1 : 0;
    }
    Check(hg_encrypt_bn(ctx, id, mag.data(), neg.data(), r, ct.data(), n));
  }
  return ct;
}

}  // namespace detail

class KeyGenerator {
 public:
  // key_generator.cc:26-60 on the engine's host code, seeded from the OS
  static void Generate(size_t key_size, SecretKey* sk, PublicKey* pk) {
    Generate(key_size, std::random_device{}() ^ ((uint64_t)std::random_device{}() << 32), sk, pk);
  }
  static void Generate(SecretKey* sk, PublicKey* pk) { Generate(2048, sk, pk); }
  // reproducible form: every random draw from the seeded stream
  static void Generate(size_t key_size, uint64_t seed, SecretKey* sk, PublicKey* pk) {
    if (key_size % 2 != 0) throw std::invalid_argument("Key size must be even");
    const size_t bits = key_size;
    std::vector<uint32_t> n(bits / 32), p(bits / 64), q(bits / 64), hs(bits / 16);
    detail::Check(hg_keygen((uint32_t)bits, seed, n.data(), p.data(), q.data(), hs.data()));
    pk->n_ = BigInt::FromMag(detail::FromLimbs(n.data(), n.size()), false);
    pk->h_s_ = BigInt::FromMag(detail::FromLimbs(hs.data(), hs.size()), false);
    pk->Init();
    sk->p_ = BigInt::FromMag(detail::FromLimbs(p.data(), p.size()), false);
    sk->q_ = BigInt::FromMag(detail::FromLimbs(q.data(), q.size()), false);
    const hg::BN lam = ((sk->p_.Mag() - hg::BN(1)) * (sk->q_.Mag() - hg::BN(1))) / hg::BN(2);
    sk->lambda_ = BigInt::FromMag(lam, false);
    sk->mu_ = BigInt::FromMag(hg::BN::invmod(lam, pk->n_.Mag()), false);
  }
};

// vector_encryptor.h:24-33
class Encryptor {
 public:
  explicit Encryptor(const PublicKey& pk) : pk_(pk) {}

  std::vector<Ciphertext> EncryptZero(int64_t size) const {
    const auto r = detail::DrawR(pk_, (size_t)size);
    std::vector<uint32_t> ct((size_t)size * pk_.Limbs());
    detail::Check(hg_encrypt_zero(detail::Engine::Get().ctx, detail::KeyId(pk_, nullptr), r.data(), ct.data(),
                                  (size_t)size));
    return detail::ToCts(pk_, ct);
  }

  std::vector<Ciphertext> Encrypt(ConstSpan<Plaintext> pts) const {
    detail::CheckPlaintexts(pk_, pts);
    const auto r = detail::DrawR(pk_, pts.size());
    return detail::ToCts(pk_, detail::EncryptLimbs(pk_, pts, r.data()));
  }

  // encryptor.cc:51-53 audit string: "p:{m},rn:{h_s^r},c:{c}"
  std::pair<std::vector<Ciphertext>, std::vector<std::string>> EncryptWithAudit(ConstSpan<Plaintext> pts) const {
    detail::CheckPlaintexts(pk_, pts);
    const auto r = detail::DrawR(pk_, pts.size());
    auto cts = detail::ToCts(pk_, detail::EncryptLimbs(pk_, pts, r.data()));
    std::vector<uint32_t> rn(pts.size() * pk_.Limbs());
    detail::Check(hg_encrypt_zero(detail::Engine::Get().ctx, detail::KeyId(pk_, nullptr), r.data(), rn.data(),
                                  pts.size()));
    const auto rns = detail::ToCts(pk_, rn);
    std::vector<std::string> audit;
    for (size_t i = 0; i < pts.size(); ++i)
      audit.push_back("p:" + pts[i]->ToHexString() + ",rn:" + rns[i].c_.ToHexString() + ",c:" +
                      cts[i].c_.ToHexString());
    return {std::move(cts), std::move(audit)};
  }

 private:
  PublicKey pk_;
};

// vector_decryptor.h:25-31
class Decryptor {
 public:
  Decryptor(const PublicKey& pk, const SecretKey& sk) : pk_(pk), sk_(sk) {
    if (sk_.p_ * sk_.q_ != pk_.n_) throw std::invalid_argument("pk and sk are not paired");
  }

  std::vector<Plaintext> Decrypt(ConstSpan<Ciphertext> cts) const {
    const size_t n = cts.size(), S = pk_.Limbs();
    const auto c = detail::CtLimbs(pk_, cts);
    std::vector<uint32_t> mag(n * (S / 2));
    std::vector<uint8_t> neg(n);
    detail::Check(hg_decrypt_bn(detail::Engine::Get().ctx, detail::KeyId(pk_, &sk_), c.data(), mag.data(),
                                neg.data(), n));
    std::vector<Plaintext> out(n);
    for (size_t i = 0; i < n; ++i) out[i] = BigInt::FromMag(detail::FromLimbs(&mag[i * (S / 2)], S / 2), neg[i] != 0);
    return out;
  }

  void Decrypt(ConstSpan<Ciphertext> in_cts, Span<Plaintext> out_pts) const {
    auto res = Decrypt(in_cts);
    for (size_t i = 0; i < res.size(); ++i) *out_pts[i] = std::move(res[i]);
  }

 private:
  PublicKey pk_;
  SecretKey sk_;
};

// vector_evaluator.h:24-66, plus the optional ReduceSum hook that numpy
// MatMul detects (numpy/evaluator.cc:250-260).
class Evaluator {
 public:
  explicit Evaluator(const PublicKey& pk) : pk_(pk) {}

  void Randomize(Span<Ciphertext> cts) const {
    std::vector<const Ciphertext*> in(cts.begin(), cts.end());
    auto c = detail::CtLimbs(pk_, ConstSpan<Ciphertext>(in));
    const auto r = detail::DrawR(pk_, cts.size());
    detail::Check(hg_randomize(ctx(), id(), c.data(), r.data(), cts.size()));
    auto out = detail::ToCts(pk_, c);
    for (size_t i = 0; i < cts.size(); ++i) *cts[i] = std::move(out[i]);
  }

  std::vector<Ciphertext> Add(ConstSpan<Ciphertext> a, ConstSpan<Ciphertext> b) const {
    SameSize(a.size(), b.size());
    const auto x = detail::CtLimbs(pk_, a), y = detail::CtLimbs(pk_, b);
    std::vector<uint32_t> out(x.size());
    detail::Check(hg_add(ctx(), id(), x.data(), y.data(), out.data(), a.size()));
    return detail::ToCts(pk_, out);
  }
  std::vector<Ciphertext> Add(ConstSpan<Ciphertext> a, ConstSpan<Plaintext> b) const {
    SameSize(a.size(), b.size());
    const auto x = detail::CtLimbs(pk_, a);
    std::vector<uint32_t> out(x.size());
    for (auto* p : b)
      if (p->CompareAbs(pk_.PlaintextBound()) > 0) throw std::invalid_argument("plaintext out of range");
    if (detail::AllInt64(b)) {
      std::vector<int64_t> p(b.size());
      for (size_t i = 0; i < b.size(); ++i) p[i] = b[i]->Get<int64_t>();
      detail::Check(hg_add_plain(ctx(), id(), x.data(), p.data(), out.data(), a.size()));
    } else {
      // (1 + p*n) in Montgomery form is the encryption of p with r = 0
      const std::vector<uint32_t> r0(b.size() * (pk_.KeyBits() / 64), 0);
      const auto g = detail::EncryptLimbs(pk_, b, r0.data());
      detail::Check(hg_add(ctx(), id(), x.data(), g.data(), out.data(), a.size()));
    }
    return detail::ToCts(pk_, out);
  }
  std::vector<Ciphertext> Add(ConstSpan<Plaintext> a, ConstSpan<Ciphertext> b) const { return Add(b, a); }
  std::vector<Plaintext> Add(ConstSpan<Plaintext> a, ConstSpan<Plaintext> b) const {
    SameSize(a.size(), b.size());
    std::vector<Plaintext> out(a.size());
    for (size_t i = 0; i < a.size(); ++i) out[i] = *a[i] + *b[i];
    return out;
  }

  void AddInplace(Span<Ciphertext> a, ConstSpan<Ciphertext> b) const { Assign(a, Add(Const(a), b)); }
  void AddInplace(Span<Ciphertext> a, ConstSpan<Plaintext> b) const { Assign(a, Add(Const(a), b)); }
  void AddInplace(Span<Plaintext> a, ConstSpan<Plaintext> b) const { AssignP(a, Add(ConstP(a), b)); }

  // evaluator.cc:66-84
  std::vector<Ciphertext> Sub(ConstSpan<Ciphertext> a, ConstSpan<Ciphertext> b) const {
    SameSize(a.size(), b.size());
    const auto x = detail::CtLimbs(pk_, a), y = detail::CtLimbs(pk_, b);
    std::vector<uint32_t> out(x.size());
    detail::Check(hg_sub(ctx(), id(), x.data(), y.data(), out.data(), a.size()));
    return detail::ToCts(pk_, out);
  }
  std::vector<Ciphertext> Sub(ConstSpan<Ciphertext> a, ConstSpan<Plaintext> b) const {
    std::vector<Plaintext> neg(b.size());
    std::vector<const Plaintext*> pn(b.size());
    for (size_t i = 0; i < b.size(); ++i) {
      neg[i] = -*b[i];
      pn[i] = &neg[i];
    }
    return Add(a, ConstSpan<Plaintext>(pn));
  }
  std::vector<Ciphertext> Sub(ConstSpan<Plaintext> a, ConstSpan<Ciphertext> b) const {
    auto nb = Negate(b);
    std::vector<const Ciphertext*> p(nb.size());
    for (size_t i = 0; i < nb.size(); ++i) p[i] = &nb[i];
    return Add(ConstSpan<Ciphertext>(p), a);
  }
  std::vector<Plaintext> Sub(ConstSpan<Plaintext> a, ConstSpan<Plaintext> b) const {
    SameSize(a.size(), b.size());
    std::vector<Plaintext> out(a.size());
    for (size_t i = 0; i < a.size(); ++i) out[i] = *a[i] - *b[i];
    return out;
  }
  void SubInplace(Span<Ciphertext> a, ConstSpan<Ciphertext> b) const { Assign(a, Sub(Const(a), b)); }
  void SubInplace(Span<Ciphertext> a, ConstSpan<Plaintext> b) const { Assign(a, Sub(Const(a), b)); }
  void SubInplace(Span<Plaintext> a, ConstSpan<Plaintext> b) const { AssignP(a, Sub(ConstP(a), b)); }

  // evaluator.cc:99-123: scalars of any size up to the width of n^2 (int64
  // scalars take hg_mul, wider ones hg_mul_bn)
  std::vector<Ciphertext> Mul(ConstSpan<Ciphertext> a, ConstSpan<Plaintext> b) const {
    SameSize(a.size(), b.size());
    const auto x = detail::CtLimbs(pk_, a);
    std::vector<uint32_t> out(x.size());
    size_t bits = 0;
    bool fits = true;
    for (size_t i = 0; i < b.size(); ++i) {
      bits = std::max(bits, b[i]->BitCount());
      fits &= b[i]->BitCount() <= 63 ||
              (b[i]->IsNegative() && b[i]->BitCount() == 64 && b[i]->Mag() == hg::BN(1ull << 63));
    }
    if (fits) {
      std::vector<int64_t> k(b.size());
      for (size_t i = 0; i < b.size(); ++i) k[i] = b[i]->Get<int64_t>();
      detail::Check(hg_mul(ctx(), id(), x.data(), k.data(), out.data(), a.size()));
    } else {
      const size_t kl = (bits + 31) / 32;
      if (kl > pk_.Limbs()) throw std::invalid_argument("GB300 Paillier: scalar wider than n^2");
      std::vector<uint32_t> mag(b.size() * kl);
      std::vector<uint8_t> neg(b.size());
      for (size_t i = 0; i < b.size(); ++i) {
        b[i]->Mag().to_limbs(mag.data() + i * kl, kl);
        neg[i] = b[i]->IsNegative() ? 1 : 0;
      }
      detail::Check(hg_mul_bn(ctx(), id(), x.data(), mag.data(), neg.data(), kl, out.data(), a.size()));
    }
    return detail::ToCts(pk_, out);
  }
  std::vector<Ciphertext> Mul(ConstSpan<Plaintext> a, ConstSpan<Ciphertext> b) const { return Mul(b, a); }
  std::vector<Plaintext> Mul(ConstSpan<Plaintext> a, ConstSpan<Plaintext> b) const {
    SameSize(a.size(), b.size());
    std::vector<Plaintext> out(a.size());
    for (size_t i = 0; i < a.size(); ++i) out[i] = *a[i] * *b[i];
    return out;
  }
  void MulInplace(Span<Ciphertext> a, ConstSpan<Plaintext> b) const { Assign(a, Mul(Const(a), b)); }
  void MulInplace(Span<Plaintext> a, ConstSpan<Plaintext> b) const { AssignP(a, Mul(ConstP(a), b)); }

  // evaluator.cc:86-97
  std::vector<Ciphertext> Negate(ConstSpan<Ciphertext> a) const {
    const auto x = detail::CtLimbs(pk_, a);
    std::vector<uint32_t> out(x.size());
    detail::Check(hg_negate(ctx(), id(), x.data(), out.data(), a.size()));
    return detail::ToCts(pk_, out);
  }
  void NegateInplace(Span<Ciphertext> a) const { Assign(a, Negate(Const(a))); }

  Ciphertext ReduceSum(ConstSpan<Ciphertext> a) const {
    const auto x = detail::CtLimbs(pk_, a);
    std::vector<uint32_t> out(pk_.Limbs());
    detail::Check(hg_sum(ctx(), id(), x.data(), a.size(), out.data()));
    return detail::ToCts(pk_, out)[0];
  }

 private:
  static hg_ctx* ctx() { return detail::Engine::Get().ctx; }
  int id() const { return detail::KeyId(pk_, nullptr); }
  static void SameSize(size_t a, size_t b) {
    if (a != b) throw std::invalid_argument("span sizes differ");
  }
  static ConstSpan<Ciphertext> Const(Span<Ciphertext> s) {
    return ConstSpan<Ciphertext>(reinterpret_cast<const Ciphertext* const*>(s.begin()), s.size());
  }
  static ConstSpan<Plaintext> ConstP(Span<Plaintext> s) {
    return ConstSpan<Plaintext>(reinterpret_cast<const Plaintext* const*>(s.begin()), s.size());
  }
  static void Assign(Span<Ciphertext> dst, std::vector<Ciphertext> v) {
    for (size_t i = 0; i < v.size(); ++i) *dst[i] = std::move(v[i]);
  }
  static void AssignP(Span<Plaintext> dst, std::vector<Plaintext> v) {
    for (size_t i = 0; i < v.size(); ++i) *dst[i] = std::move(v[i]);
  }
  PublicKey pk_;
};

}  // namespace heu::lib::algorithms::paillier_gb300

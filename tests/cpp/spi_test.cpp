// Exercises the C++ SPI adapter (heu_gb300/cpp/paillier_gb300.h) the way
// HEU's own paillier_zahlen tests drive a schema (zpaillier_test.cc:
// encrypt/decrypt round trips, homomorphic add/sub/mul/negate, plaintext
// range errors), and prints every ciphertext it makes so that the caller can
// compare them bit for bit with the oracle under the same seeded r stream.
//
//   spi_test keygen <bits> <seed>          key only (no GPU needed)
//   spi_test full <bits> <seed> <r_seed>   every SPI call (GPU)
//
// Output: one "name value" line per item (hex values), then "OK" last.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../heu_gb300/cpp/paillier_gb300.h"

namespace hea = heu::lib::algorithms;
namespace pg = heu::lib::algorithms::paillier_gb300;

static int g_fail = 0;
#define EXPECT(cond)                                                   \
  do {                                                                 \
    if (!(cond)) {                                                     \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #cond);       \
      ++g_fail;                                                        \
    }                                                                  \
  } while (0)

template <typename T>
static std::vector<const T*> ptrs(const std::vector<T>& v) {
  std::vector<const T*> p;
  for (auto& x : v) p.push_back(&x);
  return p;
}
template <typename T>
static std::vector<T*> mptrs(std::vector<T>& v) {
  std::vector<T*> p;
  for (auto& x : v) p.push_back(&x);
  return p;
}

static void print_cts(const char* name, const std::vector<pg::Ciphertext>& v) {
  for (size_t i = 0; i < v.size(); ++i) std::printf("%s[%zu] %s\n", name, i, v[i].c_.ToHexString().c_str());
}

template <typename F>
static bool throws(F f) {
  try {
    f();
  } catch (const std::exception&) {
    return true;
  }
  return false;
}

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: spi_test keygen|full bits seed [r_seed]\n");
    return 2;
  }
  const std::string mode = argv[1];
  const size_t bits = std::strtoull(argv[2], nullptr, 10);
  const uint64_t seed = std::strtoull(argv[3], nullptr, 10);

  pg::SecretKey sk;
  pg::PublicKey pk;
  pg::KeyGenerator::Generate(bits, seed, &sk, &pk);
  std::printf("n %s\np %s\nq %s\nh_s %s\n", pk.n_.ToHexString().c_str(), sk.p_.ToHexString().c_str(),
              sk.q_.ToHexString().c_str(), pk.h_s_.ToHexString().c_str());
  EXPECT(sk.p_ * sk.q_ == pk.n_);
  EXPECT(pk.n_.BitCount() == bits);
  EXPECT(throws([&] { pg::KeyGenerator::Generate(bits + 1, seed, &sk, &pk); }));
  if (mode == "keygen") {
    std::printf(g_fail ? "FAILED\n" : "OK\n");
    return g_fail ? 1 : 0;
  }

  pg::SetRandomStreamForTesting(std::strtoull(argv[4], nullptr, 10));
  pg::Encryptor enc(pk);
  pg::Decryptor dec(pk, sk);
  pg::Evaluator ev(pk);

  // plaintexts: small, int64 edges, and full-range values at +-n/2
  const pg::BigInt half = pk.PlaintextBound();
  std::vector<pg::Plaintext> pts = {
      pg::BigInt(0),          pg::BigInt(1),   pg::BigInt(-1),     pg::BigInt(123456789),
      pg::BigInt(-987654321), pg::BigInt(INT64_MAX), pg::BigInt(INT64_MIN + 1),
      half,                   -half,           half - pg::BigInt(12345),
  };
  auto cts = enc.Encrypt(hea::ConstSpan<pg::Plaintext>(ptrs(pts)));
  print_cts("enc", cts);
  auto back = dec.Decrypt(hea::ConstSpan<pg::Ciphertext>(ptrs(cts)));
  for (size_t i = 0; i < pts.size(); ++i) EXPECT(back[i] == pts[i]);

  // Decrypt into caller-owned plaintexts
  std::vector<pg::Plaintext> outs(cts.size());
  dec.Decrypt(hea::ConstSpan<pg::Ciphertext>(ptrs(cts)), hea::Span<pg::Plaintext>(mptrs(outs)));
  for (size_t i = 0; i < pts.size(); ++i) EXPECT(outs[i] == pts[i]);

  // out-of-range plaintext: |m| > n/2 (encryptor.cc:36-39)
  std::vector<pg::Plaintext> bad = {half + pg::BigInt(1)};
  EXPECT(throws([&] { enc.Encrypt(hea::ConstSpan<pg::Plaintext>(ptrs(bad))); }));

  // small operands for the homomorphic checks
  std::vector<pg::Plaintext> a = {pg::BigInt(5), pg::BigInt(-7), pg::BigInt(1000000), pg::BigInt(0)};
  std::vector<pg::Plaintext> b = {pg::BigInt(11), pg::BigInt(3), pg::BigInt(-2000000), pg::BigInt(-9)};
  auto ca = enc.Encrypt(hea::ConstSpan<pg::Plaintext>(ptrs(a)));
  auto cb = enc.Encrypt(hea::ConstSpan<pg::Plaintext>(ptrs(b)));
  print_cts("ca", ca);
  print_cts("cb", cb);
  const auto pca = ptrs(ca), pcb = ptrs(cb);
  const auto ppa = ptrs(a), ppb = ptrs(b);
  const hea::ConstSpan<pg::Ciphertext> A(pca), B(pcb);
  const hea::ConstSpan<pg::Plaintext> PA(ppa), PB(ppb);
  auto D = [&](const std::vector<pg::Ciphertext>& v) { return dec.Decrypt(hea::ConstSpan<pg::Ciphertext>(ptrs(v))); };

  auto add_cc = ev.Add(A, B);
  auto add_cp = ev.Add(A, PB);
  auto add_pc = ev.Add(PA, B);
  auto sub_cc = ev.Sub(A, B);
  auto sub_cp = ev.Sub(A, PB);
  auto sub_pc = ev.Sub(PA, B);
  auto mul_cp = ev.Mul(A, PB);
  auto neg = ev.Negate(A);
  print_cts("add_cc", add_cc);
  print_cts("add_cp", add_cp);
  print_cts("sub_cc", sub_cc);
  print_cts("mul_cp", mul_cp);
  print_cts("neg", neg);
  auto dadd = D(add_cc), daddp = D(add_cp), daddpc = D(add_pc), dsub = D(sub_cc), dsubp = D(sub_cp),
       dsubpc = D(sub_pc), dmul = D(mul_cp), dneg = D(neg);
  for (size_t i = 0; i < a.size(); ++i) {
    EXPECT(dadd[i] == a[i] + b[i]);
    EXPECT(daddp[i] == a[i] + b[i]);
    EXPECT(daddpc[i] == a[i] + b[i]);
    EXPECT(dsub[i] == a[i] - b[i]);
    EXPECT(dsubp[i] == a[i] - b[i]);
    EXPECT(dsubpc[i] == a[i] - b[i]);
    EXPECT(dmul[i] == a[i] * b[i]);
    EXPECT(dneg[i] == -a[i]);
  }

  // full-range plaintext addend goes through the encrypt-with-r=0 path
  std::vector<pg::Plaintext> big = {half - pg::BigInt(100), -half + pg::BigInt(100), pg::BigInt(1), pg::BigInt(2)};
  auto add_big = D(ev.Add(A, hea::ConstSpan<pg::Plaintext>(ptrs(big))));
  EXPECT(add_big[0] == a[0] + big[0]);
  EXPECT(add_big[1] == a[1] + big[1]);

  // plaintext-plaintext arithmetic stays on the host
  auto pp = ev.Mul(PA, PB);
  for (size_t i = 0; i < a.size(); ++i) EXPECT(pp[i] == a[i] * b[i]);

  // in-place forms
  auto ia = ca;
  ev.AddInplace(hea::Span<pg::Ciphertext>(mptrs(ia)), B);
  EXPECT(ia == add_cc);
  ia = ca;
  ev.SubInplace(hea::Span<pg::Ciphertext>(mptrs(ia)), B);
  EXPECT(ia == sub_cc);
  ia = ca;
  ev.MulInplace(hea::Span<pg::Ciphertext>(mptrs(ia)), PB);
  EXPECT(ia == mul_cp);
  ia = ca;
  ev.NegateInplace(hea::Span<pg::Ciphertext>(mptrs(ia)));
  EXPECT(ia == neg);

  // Randomize keeps the plaintext and changes the ciphertext
  auto rnd = ca;
  ev.Randomize(hea::Span<pg::Ciphertext>(mptrs(rnd)));
  auto drnd = D(rnd);
  for (size_t i = 0; i < a.size(); ++i) {
    EXPECT(drnd[i] == a[i]);
    EXPECT(rnd[i] != ca[i]);
  }

  // EncryptZero and EncryptWithAudit
  auto zeros = enc.EncryptZero(3);
  for (auto& z : D(zeros)) EXPECT(z.IsZero());
  auto audited = enc.EncryptWithAudit(PA);
  EXPECT(audited.second.size() == a.size());
  EXPECT(audited.second[0].rfind("p:5,rn:", 0) == 0);
  for (size_t i = 0; i < a.size(); ++i)
    EXPECT(audited.second[i].find(",c:" + audited.first[i].c_.ToHexString()) != std::string::npos);
  for (auto& s : audited.second) std::printf("audit %s\n", s.c_str());

  // ReduceSum (the numpy MatMul hook)
  auto rs = ev.ReduceSum(A);
  std::printf("sum %s\n", rs.c_.ToHexString().c_str());
  EXPECT(dec.Decrypt(hea::ConstSpan<pg::Ciphertext>(std::vector<const pg::Ciphertext*>{&rs}))[0] ==
         a[0] + a[1] + a[2] + a[3]);

  // a HEU build whose yacl backend keeps Montgomery residues in another
  // radix (libtommath: 60-bit digits) exchanges ciphertexts in that radix
  pg::PublicKey pk60 = pk;
  const size_t radix60 = 60 * ((pk.n_square_.BitCount() + 59) / 60);
  pk60.SetBackendRadixBits(radix60);
  pg::Encryptor enc60(pk60);
  pg::Decryptor dec60(pk60, sk);
  pg::Evaluator ev60(pk60);
  auto c60 = enc60.Encrypt(PA);
  print_cts("radix60", c60);
  std::printf("radix60_bits %zu\n", radix60);
  auto d60 = dec60.Decrypt(hea::ConstSpan<pg::Ciphertext>(ptrs(c60)));
  auto s60 = dec60.Decrypt(hea::ConstSpan<pg::Ciphertext>(ptrs(ev60.Add(hea::ConstSpan<pg::Ciphertext>(ptrs(c60)),
                                                                           hea::ConstSpan<pg::Ciphertext>(ptrs(c60))))));
  for (size_t i = 0; i < a.size(); ++i) {
    EXPECT(d60[i] == a[i]);
    EXPECT(s60[i] == a[i] + a[i]);
  }

  // scalars wider than int64 (evaluator.cc:99-123 takes any BigInt)
  std::vector<pg::Plaintext> wide = {half, -half, pg::BigInt(1) - half, pg::BigInt::FromHex("10000000000000000")};
  auto mul_big = ev.Mul(A, hea::ConstSpan<pg::Plaintext>(ptrs(wide)));
  print_cts("mul_big", mul_big);

  // errors: mismatched spans, scalar wider than n^2, unpaired key
  EXPECT(throws([&] { ev.Add(A, hea::ConstSpan<pg::Ciphertext>(ptrs(std::vector<pg::Ciphertext>(ca.begin(), ca.begin() + 2)))); }));
  std::vector<pg::Plaintext> huge = {pg::BigInt::FromMag(pk.n_square_.Mag() * pk.n_square_.Mag(), false)};
  EXPECT(throws([&] { ev.Mul(hea::ConstSpan<pg::Ciphertext>(std::vector<const pg::Ciphertext*>{&ca[0]}),
                             hea::ConstSpan<pg::Plaintext>(ptrs(huge))); }));
  pg::SecretKey sk2;
  pg::PublicKey pk2;
  pg::KeyGenerator::Generate(bits, seed + 1, &sk2, &pk2);
  EXPECT(throws([&] { pg::Decryptor bad_pair(pk, sk2); }));
  // a ciphertext outside [0, n^2) is rejected by the engine
  pg::Ciphertext oob(pk.n_square_ + pg::BigInt(1));
  EXPECT(throws([&] { dec.Decrypt(hea::ConstSpan<pg::Ciphertext>(std::vector<const pg::Ciphertext*>{&oob})); }));

  std::printf(g_fail ? "FAILED\n" : "OK\n");
  return g_fail ? 1 : 0;
}

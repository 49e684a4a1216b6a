// Host big-number code (heu_gb300/csrc/host_bn.hpp) under AddressSanitizer
// and UndefinedBehaviorSanitizer: key generation and the batch-inverse root
// depend on it.  Prints one line per case: op, operands, result (hex); the
// Python side recomputes every result with Python integers.
#include <cstdio>
#include <string>
#include <vector>

#include "../../heu_gb300/csrc/host_bn.hpp"

using hg::BN;

static std::string hex(const BN& v) {
  if (v.is_zero()) return "0";
  std::string s;
  static const char* dig = "0123456789abcdef";
  for (size_t i = v.d.size(); i-- > 0;)
    for (int b = 28; b >= 0; b -= 4) s.push_back(dig[(v.d[i] >> b) & 0xf]);
  return s.substr(s.find_first_not_of('0'));
}

int main() {
  hg::Xoshiro prg(2024);
  const size_t sizes[] = {1, 31, 32, 33, 64, 95, 512, 1024, 2048, 4096};
  for (size_t bits_a : sizes) {
    for (size_t bits_b : sizes) {
      BN a = prg.randbits(bits_a), b = prg.randbits(bits_b);
      if (b.is_zero()) b = BN(7);
      std::printf("add %s %s %s\n", hex(a).c_str(), hex(b).c_str(), hex(a + b).c_str());
      if (a >= b) std::printf("sub %s %s %s\n", hex(a).c_str(), hex(b).c_str(), hex(a - b).c_str());
      std::printf("mul %s %s %s\n", hex(a).c_str(), hex(b).c_str(), hex(a * b).c_str());
      BN q, r;
      BN::divmod(a, b, &q, &r);
      std::printf("divmod %s %s %s %s\n", hex(a).c_str(), hex(b).c_str(), hex(q).c_str(), hex(r).c_str());
      std::printf("shl %s %zu %s\n", hex(a).c_str(), bits_b % 97, hex(a.shl(bits_b % 97)).c_str());
      std::printf("shr %s %zu %s\n", hex(a).c_str(), bits_b % 97, hex(a.shr(bits_b % 97)).c_str());
    }
  }
  // modular inverse, power and Montgomery power on odd moduli
  for (size_t bits : {64, 512, 1024, 2048, 4096}) {
    for (int t = 0; t < 3; ++t) {
      BN m = prg.randbits(bits);
      m.d.resize((bits + 31) / 32, 0);
      m.d[0] |= 1u;
      m.d[(bits - 1) / 32] |= 1u << ((bits - 1) % 32);
      m.trim();
      BN x = prg.randbits(bits - 1), e = prg.randbits(160);
      if (BN::gcd(x, m) == BN(1))
        std::printf("invmod %s %s %s\n", hex(x).c_str(), hex(m).c_str(), hex(BN::invmod(x, m)).c_str());
      std::printf("powmod %s %s %s %s\n", hex(x).c_str(), hex(e).c_str(), hex(m).c_str(),
                  hex(BN::powmod(x, e, m)).c_str());
      hg::HostMont mont(m);
      std::printf("montpow %s %s %s %s\n", hex(x).c_str(), hex(e).c_str(), hex(m).c_str(),
                  hex(mont.pow(x, e)).c_str());
      // root inverse on S 32-bit limbs with R = 2^(32 S): returns X^-1 R given X R
      const size_t S = (bits + 31) / 32;
      std::vector<uint32_t> xr(S), out(S);
      const BN R = BN(1).shl(32 * S);
      const BN xm = (x * (R % m)) % m;
      xm.to_limbs(xr.data(), S);
      if (hg::mont_root_inverse(xr.data(), m, S, out.data()))
        std::printf("rootinv %s %s %zu %s\n", hex(x).c_str(), hex(m).c_str(), S,
                    hex(BN::from_limbs(out.data(), S)).c_str());
    }
  }
  std::printf("OK\n");
  return 0;
}

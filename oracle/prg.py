"""Seeded pseudo-random streams shared by the oracle, the tests and the bench.

TEST INFRASTRUCTURE ONLY. Nothing in the shipped engine imports this module.

The reference draws its randomness from yacl's RNG (`BigInt::RandomExactBits`,
`RandomLtN`, `RandPrimeOver`), which cannot be seeded or reproduced outside
yacl. Parity therefore injects the same explicit stream into the oracle and
into the engine.  The generator is xoshiro256** (Blackman & Vigna, 2018)
seeded by SplitMix64 (Steele, Lea & Flood, 2014); both are published
algorithms, restated here and, identically, in the engine's host C++
(`heu_gb300/csrc/host_bn.hpp`) so that key generation from a seed agrees.

Conventions:
  * ``randbits(k)`` concatenates ceil(k/64) outputs little-endian (first
    output = least significant 64 bits) and masks to k bits.  This is the
    stand-in for ``BigInt::RandomExactBits(k)`` (uniform in [0, 2^k)).
  * ``below(n)`` rejection-samples ``randbits(bitlen(n))`` until < n
    (stand-in for ``BigInt::RandomLtN``).
"""

MASK64 = (1 << 64) - 1


def splitmix64(state):
    """One SplitMix64 step: returns (new_state, output)."""
    state = (state + 0x9E3779B97F4A7C15) & MASK64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return state, z ^ (z >> 31)


def _rotl(x, k):
    return ((x << k) | (x >> (64 - k))) & MASK64


class Prg:
    """xoshiro256** seeded from a 64-bit seed through SplitMix64."""

    def __init__(self, seed):
        st = seed & MASK64
        s = []
        for _ in range(4):
            st, out = splitmix64(st)
            s.append(out)
        self.s = s

    def next_u64(self):
        s = self.s
        result = (_rotl((s[1] * 5) & MASK64, 7) * 9) & MASK64
        t = (s[1] << 17) & MASK64
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = _rotl(s[3], 45)
        return result

    def randbits(self, k):
        if k <= 0:
            return 0
        words = (k + 63) // 64
        v = 0
        for i in range(words):
            v |= self.next_u64() << (64 * i)
        return v & ((1 << k) - 1)

    def below(self, n):
        if n <= 0:
            raise ValueError("below(n) needs n > 0")
        k = n.bit_length()
        while True:
            v = self.randbits(k)
            if v < n:
                return v

    def int64_uniform(self, lo, hi):
        """Uniform integer in [lo, hi) (hi - lo <= 2^64)."""
        span = hi - lo
        return lo + self.below(span)

    def u01(self):
        """Uniform double in [0, 1) from the top 53 bits of one output."""
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))

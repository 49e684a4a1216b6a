"""Definitional CPU oracle for HEU's Okamoto-Uchiyama scheme (`ou`).

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` and ``bench.py``'s CPU
baseline leg as the checker, never by the shipped engine.

Every function restates the reference's algorithm with Python integers and
cites the reference line it follows (paths relative to the HEU project root):

  key generation   heu/library/algorithms/ou/key_generator.cc:26-96
  public key init  heu/library/algorithms/ou/public_key.cc:28-41
  random bits      heu/library/algorithms/ou/public_key.h:27-31
  encrypt          heu/library/algorithms/ou/encryptor.cc:25-33, 92-117
  decrypt          heu/library/algorithms/ou/decryptor.cc:21-45
  evaluator        heu/library/algorithms/ou/evaluator.cc:21-125

Representation.  ``Ciphertext::c_`` lives in yacl's Montgomery space over n
(encryptor.cc:112-113; decryptor.cc:31 maps it back).  n = p^2 q has
2049-2052 bits for a 2048-bit key; the engine computes over 128 32-bit limbs
(64 for 1024-bit keys), so this oracle states the radix as R = 2^(32*S) with
those S (``limbs_for``).  Values are the
canonical Z-form c in [0, n) unless a name says ``mont``; Z-forms are unique
given the key and r.

Randomness.  Key generation draws from the project PRG (``oracle.prg``) in
place of yacl's RNG: RandPrimeOver(b) -> a b-bit odd prime (top bit set,
``is_probable_prime``), RandomMonicExactBits(b) -> randbits(b) | 2^(b-1),
RandomLtN(n) -> below(n).  Encryption randomness r (RandomExactBits of 110
bits for a 2048-bit key, encryptor.cc:12-33) is an explicit argument.
"""

from math import gcd

from oracle.paillier_z import PaillierError, is_probable_prime
from oracle.prg import Prg


def limbs_for(n_bits):
    """32-bit limbs of the engine's Montgomery radix over n: 64 for 1024-bit
    keys (n of ~1030 bits), 128 for 2048 / 3072 (n of ~2052 / ~3078 bits)."""
    return 64 if n_bits <= 2048 else 128


def random_bits_for(n_bits):
    """encryptor.cc:12-20 with public_key.h:27-31 (80 / 110 / 128 bits)."""
    if n_bits >= 2560:
        return 128
    if n_bits >= 1536:
        return 110
    return 80


def rand_prime(prg, bits):
    while True:
        c = prg.randbits(bits) | (1 << (bits - 1)) | 1
        if is_probable_prime(c):
            return c


class PublicKey:
    def __init__(self, n, G, H, max_plaintext):
        self.n = n
        self.G = G
        self.H = H
        self.G_inv = pow(G, -1, n)  # public_key.cc:29
        self.max_plaintext = max_plaintext
        self.key_size = n.bit_length()
        self.S = limbs_for(self.key_size)
        self.R = 1 << (32 * self.S)
        self.random_bits = random_bits_for(self.key_size)


class SecretKey:
    def __init__(self, p, q, t, gp_inv):
        self.p = p
        self.q = q
        self.t = t
        self.gp_inv = gp_inv
        self.p2 = p * p
        self.p_half = p >> 1
        self.n = self.p2 * q


def keygen(key_size, seed):
    """key_generator.cc:26-96 with every random draw from Prg(seed)."""
    prg = Prg(seed)
    secret_size = (key_size + 2) // 3
    if key_size >= 3072:
        pf_size = 256
    elif key_size >= 2048:
        pf_size = 224
    else:
        pf_size = 160
    if pf_size * 2 > secret_size:
        raise PaillierError(f"Key size must be larger than {pf_size * 2 * 3 - 2} bits")
    u_bits = secret_size - pf_size + 2
    while True:
        t = rand_prime(prg, pf_size)
        u = prg.randbits(u_bits) | (1 << (u_bits - 1))
        p = t * u + 1
        if is_probable_prime(p):
            break
    q = rand_prime(prg, secret_size + 1)
    p2 = p * p
    n = p2 * q
    while True:
        while True:
            g = prg.below(n)
            if gcd(g, p) == 1:
                break
        gp = pow(g % p2, p - 1, p2)
        if pow(gp, p, p2) == 1:
            break
    gp_inv = pow((gp - 1) // p, -1, p)
    while True:
        g_ = prg.below(n)
        if g_ % p != 0:
            break
    G = pow(g, u, n)
    H = pow(g_, n * u, n)
    max_plaintext = 1 << ((p >> 1).bit_length() - 1)
    return PublicKey(n, G, H, max_plaintext), SecretKey(p, q, t, gp_inv)


def to_mont(pk, c):
    return c * pk.R % pk.n


def from_mont(pk, cm):
    return cm * pow(pk.R, -1, pk.n) % pk.n


def _check_pt(pk, m):
    if abs(m) > pk.max_plaintext:
        raise PaillierError("message number out of range")


def _check_ct(pk, c):
    if not 0 <= c < pk.n:
        raise PaillierError("Invalid ciphertext")


def get_hr(pk, r):
    """H^r mod n (encryptor.cc:25-33 without the cache)."""
    return pow(pk.H, r, pk.n)


def g_pow(pk, m):
    """G^m, or G_inv^|m| for negative m (encryptor.cc:99-104)."""
    return pow(pk.G, m, pk.n) if m >= 0 else pow(pk.G_inv, -m, pk.n)


def encrypt(pk, m, r):
    """encryptor.cc:92-117: c = H^r * G^m mod n."""
    _check_pt(pk, m)
    return get_hr(pk, r) * g_pow(pk, m) % pk.n


def encrypt_zero(pk, r):
    return get_hr(pk, r)


def decrypt(pk, sk, c):
    """decryptor.cc:27-45."""
    _check_ct(pk, c)
    x = pow(c % sk.p2, sk.t, sk.p2) - 1
    m = (x // sk.p) * sk.gp_inv % sk.p
    if m > sk.p_half:
        m -= sk.p
    return m


def add(pk, a, b):
    _check_ct(pk, a)
    _check_ct(pk, b)
    return a * b % pk.n


def add_plain(pk, a, p):
    """evaluator.cc:35-50."""
    _check_ct(pk, a)
    _check_pt(pk, p)
    return a * g_pow(pk, p) % pk.n


def negate(pk, a):
    """evaluator.cc:76-84: a^-1 mod n."""
    _check_ct(pk, a)
    return pow(a, -1, pk.n)


def sub(pk, a, b):
    return add(pk, a, negate(pk, b))


def mul(pk, a, k):
    """evaluator.cc:88-111: k = 0 -> identity, +-1 -> a / Negate(a), else
    PowMod (negative k through the inverse)."""
    _check_ct(pk, a)
    if k == 0:
        return 1
    if k == 1:
        return a
    if k == -1:
        return negate(pk, a)
    if k < 0:
        return pow(pow(a, -1, pk.n), -k, pk.n)
    return pow(a, k, pk.n)


def randomize(pk, a, r):
    """evaluator.cc:11-14: a * H^r."""
    _check_ct(pk, a)
    return a * get_hr(pk, r) % pk.n

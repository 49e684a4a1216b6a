"""Definitional CPU oracle for HEU's ZPaillier (`paillier_z`) scheme.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` leg of ``bench.py`` as the checker, never by the
shipped engine.

Every function restates the reference's algorithm with Python integers and
cites the reference line it follows (paths relative to the HEU project root):

  key generation   heu/library/algorithms/paillier_zahlen/key_generator.cc:26-60
  secret key init  heu/library/algorithms/paillier_zahlen/secret_key.cc:19-62
  public key init  heu/library/algorithms/paillier_zahlen/public_key.cc:28-40
  encrypt          heu/library/algorithms/paillier_zahlen/encryptor.cc:26-56
  decrypt          heu/library/algorithms/paillier_zahlen/decryptor.cc:21-53
  evaluator        heu/library/algorithms/paillier_zahlen/evaluator.cc:21-127
  numpy Sum        heu/library/numpy/evaluator.cc:355-373
  numpy MatMul     heu/library/numpy/evaluator.cc:208-353
  bucket sum       heu/library/numpy/evaluator.cc:378-458, evaluator.h:84-87

Representation.  The reference keeps ``Ciphertext::c_`` in yacl's Montgomery
space over n^2 (encryptor.cc:46-49; decryptor.cc:35-36 maps it back).  yacl
is not vendored, so its radix is not visible; this oracle states it as
R = 2^(32*S) with S = 2*ceil(bitlen(n)/32) 32-bit limbs, i.e. R = 2^(2k) for a
k-bit key (the word-aligned radix that a 32- or 64-bit-word Montgomery
context over a 2k-bit modulus uses).  All values below are the canonical
Z-form c in [0, n^2) unless a name says ``mont``; the Montgomery view is
``to_mont(c) = c*R mod n^2``.  Every Z-form result is unique given the key and
the injected r, independent of yacl's table layout or exponentiation order.

Randomness.  ``Encryptor::GetRn`` draws r = RandomExactBits(k/2)
(encryptor.cc:26-31).  Here r is always an explicit argument: the same r
stream (``oracle.prg``) is injected into the oracle and into the engine.
"""

from math import gcd

from oracle.prg import Prg

# --------------------------------------------------------------------------
# primality (stand-in for yacl BigInt::RandPrimeOver(bits, PrimeType::BBS))
# --------------------------------------------------------------------------


def _small_primes(limit):
    sieve = bytearray([1]) * limit
    sieve[0:2] = b"\x00\x00"
    for i in range(2, int(limit ** 0.5) + 1):
        if sieve[i]:
            sieve[i * i::i] = bytearray(len(sieve[i * i::i]))
    return [i for i in range(limit) if sieve[i]]


SMALL_PRIMES = _small_primes(2000)
MR_BASES = SMALL_PRIMES[:20]  # 2, 3, 5, ..., 71


def is_probable_prime(c):
    """Trial division by primes < 2000, then Miller-Rabin to the bases 2..71."""
    if c < 2:
        return False
    for sp in SMALL_PRIMES:
        if c == sp:
            return True
        if c % sp == 0:
            return False
    d = c - 1
    s = 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in MR_BASES:
        x = pow(a, d, c)
        if x == 1 or x == c - 1:
            continue
        for _ in range(s - 1):
            x = x * x % c
            if x == c - 1:
                break
        else:
            return False
    return True


def rand_prime_bbs(prg, bits):
    """A `bits`-bit prime p = 3 (mod 4) (a Blum prime, yacl's PrimeType::BBS).

    Candidates are ``randbits(bits) | 2^(bits-1) | 3`` drawn afresh from the
    stream until one passes ``is_probable_prime``.
    """
    while True:
        c = prg.randbits(bits) | (1 << (bits - 1)) | 3
        if is_probable_prime(c):
            return c


# --------------------------------------------------------------------------
# keys
# --------------------------------------------------------------------------


def limbs_for(bits):
    return (bits + 31) // 32


class PublicKey:
    """public_key.cc:28-40: n, n^2, n/2, h_s, key_size = bitlen(n)."""

    def __init__(self, n, h_s):
        self.n = n
        self.h_s = h_s
        self.n2 = n * n
        self.n_half = n >> 1
        self.key_size = n.bit_length()
        self.S = 2 * limbs_for(self.key_size)  # 32-bit limbs of n^2
        self.R = 1 << (32 * self.S)

    def plaintext_bound(self):
        return self.n_half


class SecretKey:
    """secret_key.cc:19-43 (Init) and :45-62 (PowModNSquareCrt)."""

    def __init__(self, p, q):
        self.p = p
        self.q = q
        self.lam = (p - 1) * (q - 1) // 2
        self.mu = pow(self.lam, -1, p * q)
        self.p2 = p * p
        self.q2 = q * q
        self.n2 = self.p2 * self.q2
        q2inv = pow(self.q2, -1, self.p2)
        self.q2inv_mul_q2 = q2inv * self.q2
        self.pinv_q = pow(p, -1, q)
        self.phi_p2 = p * (p - 1)
        self.phi_q2 = q * (q - 1)
        self.phi_p = p - 1
        self.phi_q = q - 1
        n = p * q
        g = n + 1
        hp = pow(g, self.phi_p, self.p2)
        hp = (hp - 1) // p
        self.hp = pow(hp, -1, p)
        hq = pow(g, self.phi_q, self.q2)
        hq = (hq - 1) // q
        self.hq = pow(hq, -1, q)

    def pow_mod_n2_crt(self, base, exp):
        pexp = exp % self.phi_p2
        qexp = exp % self.phi_q2
        pbase = base % self.p2
        qbase = base % self.q2
        pe = pow(pbase, pexp, self.p2)
        qe = pow(qbase, qexp, self.q2)
        return ((pe - qe) * self.q2inv_mul_q2 + qe) % self.n2


KPQ_DIFFERENCE_BITLEN_SUB = 2  # key_generator.cc:23


def keygen(key_size, seed):
    """key_generator.cc:26-60 with every random draw taken from Prg(seed)."""
    if key_size % 2:
        raise ValueError("Key size must be even")
    prg = Prg(seed)
    half = key_size // 2
    while True:
        p = rand_prime_bbs(prg, half)
        while True:
            q = rand_prime_bbs(prg, half)
            c = gcd(p - 1, q - 1)
            if c == 2 and abs(p - q).bit_length() >= half - KPQ_DIFFERENCE_BITLEN_SUB:
                break
        n = p * q
        if n.bit_length() >= key_size:
            break
    while True:
        x = prg.below(n)
        if gcd(x, n) == 1:
            break
    h = -(x * x % n)
    sk = SecretKey(p, q)
    h_s = sk.pow_mod_n2_crt(h, n)
    pk = PublicKey(n, h_s)
    return pk, sk


# --------------------------------------------------------------------------
# representation helpers
# --------------------------------------------------------------------------


def to_mont(pk, c):
    return c * pk.R % pk.n2


def from_mont(pk, cm):
    return cm * pow(pk.R, -1, pk.n2) % pk.n2


def to_limbs(v, nlimbs):
    """Little-endian 32-bit limbs of a non-negative integer."""
    if v < 0 or v.bit_length() > 32 * nlimbs:
        raise ValueError("value does not fit")
    return [(v >> (32 * i)) & 0xFFFFFFFF for i in range(nlimbs)]


def from_limbs(limbs):
    v = 0
    for i, w in enumerate(limbs):
        v |= int(w) << (32 * i)
    return v


def to_bytes(v, nlimbs):
    return v.to_bytes(4 * nlimbs, "little")


def from_bytes(b):
    return int.from_bytes(b, "little")


# --------------------------------------------------------------------------
# scheme operations (Z-form in, Z-form out)
# --------------------------------------------------------------------------


class PaillierError(ValueError):
    pass


def _check_pt(pk, m):
    # encryptor.cc:38-40, evaluator.cc:48-51: |m| <= n/2
    if abs(m) > pk.n_half:
        raise PaillierError("message number out of range")


def _check_ct(pk, c):
    # decryptor.cc:21-23, evaluator.cc:21-23
    if c < 0 or c >= pk.n2:
        raise PaillierError("Invalid ciphertext")


def get_rn(pk, r):
    """encryptor.cc:26-31: h_s^r mod n^2 (r injected, r < 2^(k/2))."""
    return pow(pk.h_s, r, pk.n2)


def encrypt(pk, m, r):
    """encryptor.cc:36-56: c = (1 + n*m) * h_s^r mod n^2."""
    _check_pt(pk, m)
    gm = (pk.n * m + 1) % pk.n2
    return gm * get_rn(pk, r) % pk.n2


def encrypt_zero(pk, r):
    """encryptor.cc:33: EncryptZero = GetRn()."""
    return get_rn(pk, r)


def decrypt(pk, sk, c):
    """decryptor.cc:32-53: CRT decryption over p^2 and q^2."""
    _check_ct(pk, c)
    mp = pow(c, sk.phi_p, sk.p2)
    mp = ((mp - 1) // sk.p) * sk.hp % sk.p
    mq = pow(c, sk.phi_q, sk.q2)
    mq = ((mq - 1) // sk.q) * sk.hq % sk.q
    out = (mq - mp) * sk.pinv_q % sk.q
    out = out * sk.p + mp
    if out > pk.n_half:
        out -= pk.n
    return out


def randomize(pk, c, r):
    """evaluator.cc:25-28: c * h_s^r."""
    _check_ct(pk, c)
    return c * get_rn(pk, r) % pk.n2


def add(pk, a, b):
    """evaluator.cc:30-36: Montgomery MulMod of the two residues."""
    _check_ct(pk, a)
    _check_ct(pk, b)
    return a * b % pk.n2


def add_plain(pk, a, p):
    """evaluator.cc:46-60: a * (1 + n*p) mod n^2."""
    _check_ct(pk, a)
    _check_pt(pk, p)
    return a * ((pk.n * p + 1) % pk.n2) % pk.n2


def negate(pk, a):
    """evaluator.cc:86-97: InvMod(n^2) of the Z-form value."""
    _check_ct(pk, a)
    return pow(a, -1, pk.n2)


def sub(pk, a, b):
    """evaluator.cc:66-68: Add(a, Negate(b))."""
    return add(pk, a, negate(pk, b))


def sub_plain(pk, a, p):
    """evaluator.cc:74-76: Add(a, -p)."""
    return add_plain(pk, a, -p)


def sub_plain_ct(pk, p, a):
    """evaluator.cc:82-84: Add(Negate(a), p)."""
    return add_plain(pk, negate(pk, a), p)


def mul(pk, a, k):
    """evaluator.cc:99-123: 0 -> identity, +-1 shortcuts, else c^k mod n^2.

    For k < 0 yacl's PowMod takes the inverse first, so c^k = (c^-1)^|k|.
    """
    _check_ct(pk, a)
    if k == 0:
        return 1
    if k == 1:
        return a
    if k == -1:
        return negate(pk, a)
    return pow(a, k, pk.n2)


def identity(pk):
    """Montgomery identity (evaluator.cc:105-106) in Z-form."""
    return 1


# --------------------------------------------------------------------------
# heu.numpy reductions
# --------------------------------------------------------------------------


def sum_(pk, cs):
    """numpy/evaluator.cc:355-373: product of all ciphertexts (non-empty)."""
    if len(cs) == 0:
        raise PaillierError("you cannot sum an empty tensor")
    acc = cs[0]
    for c in cs[1:]:
        acc = acc * c % pk.n2
    return acc


def bucket_sum(pk, x, order_map, bucket_num, cumsum=False):
    """numpy/evaluator.cc:378-458 (FeatureWiseBucketSum).

    x: rows x cols list of ciphertexts; order_map: rows x features bin ids.
    Returns a (features*bucket_num) x cols matrix; row f*bucket_num+b holds
    the product of x[i][col] over rows i with order_map[i][f] == b.  Empty
    buckets hold GetZero(x) = Sub(x00, x00), whose Z-form is 1
    (numpy/evaluator.h:84-87).
    """
    rows = len(x)
    if rows == 0 or len(x[0]) == 0:
        raise PaillierError("you cannot sum an empty tensor")
    cols = len(x[0])
    features = len(order_map[0])
    out = [[1] * cols for _ in range(features * bucket_num)]
    for col in range(cols):
        for f in range(features):
            sums = [1] * bucket_num
            for i in range(rows):
                b = order_map[i][f]
                sums[b] = sums[b] * x[i][col] % pk.n2
            if cumsum:
                acc = 1
                for b in range(bucket_num):
                    acc = acc * sums[b] % pk.n2
                    out[f * bucket_num + b][col] = acc
            else:
                for b in range(bucket_num):
                    out[f * bucket_num + b][col] = sums[b]
    return out


def matmul(pk, x, y):
    """numpy/evaluator.cc:208-292: out(i,j) = prod_k x(i,k)^y(k,j) mod n^2.

    x: M x K ciphertexts, y: K x N integer plaintexts.  Each term is
    ``mul`` (so y = 0 contributes the identity and y < 0 the inverse power),
    and the terms are multiplied together (AddInplace / ReduceSum).
    """
    m_rows = len(x)
    k_dim = len(y)
    n_cols = len(y[0]) if k_dim else 0
    out = []
    for i in range(m_rows):
        row = []
        for j in range(n_cols):
            acc = mul(pk, x[i][0], y[0][j])
            for k in range(1, k_dim):
                acc = acc * mul(pk, x[i][k], y[k][j]) % pk.n2
            row.append(acc)
        out.append(row)
    return out


def r_stream(seed, count, bits):
    """The injected encryption randomness: count draws of randbits(bits)."""
    prg = Prg(seed)
    return [prg.randbits(bits) for _ in range(count)]

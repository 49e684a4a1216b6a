"""The paillier_z oracle pinned against the reference's own tests.

HEU's tests are identity / round-trip checks with literal expected values
(the reference holds no ciphertext known-answer vectors); each test below
restates one of them against the oracle, citing the reference test.
"""

import json
import os
from math import gcd

import numpy as np
import pytest

from oracle import paillier_z as pz
from oracle.prg import Prg, splitmix64
from tests.conftest import oracle_key

HERE = os.path.dirname(os.path.abspath(__file__))
I64_MIN, I64_MAX = -(2 ** 63), 2 ** 63 - 1


@pytest.fixture(scope="module")
def key1024():
    return oracle_key(1024, 1)


def enc(pk, m, seed=1):
    return pz.encrypt(pk, m, pz.r_stream(seed, 1, pk.key_size // 2)[0])


def test_splitmix64_published_first_output():
    # SplitMix64 from state 0 (Steele, Lea & Flood 2014): first output
    assert splitmix64(0)[1] == 0xE220A8397B1DCDAF


def test_prg_is_deterministic():
    a, b = Prg(5), Prg(5)
    assert [a.next_u64() for _ in range(8)] == [b.next_u64() for _ in range(8)]
    assert Prg(1).randbits(1024) < 2 ** 1024
    assert Prg(6).below(1000) < 1000


@pytest.mark.parametrize("bits,seed", [(1024, 1), (2048, 0)])
def test_keygen_invariants(bits, seed):
    """key_generator_test.cc:26-40 and key_generator.cc:26-60."""
    pk, sk = oracle_key(bits, seed)
    p, q = sk.p, sk.q
    assert p % 4 == 3 and q % 4 == 3  # Blum (BBS) primes
    assert pz.is_probable_prime(p) and pz.is_probable_prime(q)
    assert gcd(p - 1, q - 1) == 2
    assert abs(p - q).bit_length() >= bits // 2 - 2
    assert pk.n == p * q and pk.n.bit_length() == bits
    assert sk.lam == (p - 1) * (q - 1) // 2
    assert sk.mu * sk.lam % pk.n == 1
    # h_s is an n-th residue: h_s^lambda = 1 mod n^2
    assert pow(pk.h_s, sk.lam, pk.n2) == 1
    assert pk.n_half == pk.n >> 1


def test_ciphertext_evaluate(key1024):
    """paillier_test.cc:40-97 (CiphertextEvaluate)."""
    pk, sk = key1024
    c0 = enc(pk, -12345, 1)
    assert pz.decrypt(pk, sk, pz.add(pk, c0, c0)) == -12345 * 2
    res = pz.mul(pk, c0, 2)
    assert pz.decrypt(pk, sk, res) == -12345 * 2
    res = pz.randomize(pk, res, 77)
    assert pz.decrypt(pk, sk, res) == -12345 * 2
    c1 = enc(pk, 123, 2)
    assert pz.decrypt(pk, sk, pz.add(pk, c1, c1)) == 246
    assert pz.decrypt(pk, sk, pz.mul(pk, c1, 2)) == 246
    assert pz.decrypt(pk, sk, pz.add(pk, c0, c1)) == -12345 + 123
    assert pz.decrypt(pk, sk, pz.mul(pk, c1, 1)) == 123
    z = pz.mul(pk, c1, 0)
    assert pz.decrypt(pk, sk, z) == 0
    z = pz.randomize(pk, z, 5)
    assert z != 0 and pz.decrypt(pk, sk, z) == 0
    assert pz.decrypt(pk, sk, pz.mul(pk, c1, -1)) == -123
    assert pz.decrypt(pk, sk, pz.mul(pk, c1, -2)) == -246


def test_min_max_decrypt(key1024):
    """paillier_test.cc:99-119 (MinMaxDecrypt)."""
    pk, sk = key1024
    with pytest.raises(pz.PaillierError):
        enc(pk, pk.n)
    with pytest.raises(pz.PaillierError):
        enc(pk, pk.plaintext_bound() + 1)
    mx = pk.plaintext_bound()
    assert pz.decrypt(pk, sk, enc(pk, mx)) == mx
    assert pz.decrypt(pk, sk, enc(pk, -mx)) == -mx
    with pytest.raises(pz.PaillierError):
        enc(pk, -mx - 1)


def test_plaintext_evaluate(key1024):
    """paillier_test.cc:121-176 (PlaintextEvaluate1/2)."""
    pk, sk = key1024
    c0 = enc(pk, 123)
    for p, want in ((23, 146), (6543212, 123 + 6543212), (-123, 0), (-456, 123 - 456)):
        assert pz.decrypt(pk, sk, pz.add_plain(pk, c0, p)) == want
    c0 = enc(pk, -123)
    for p, want in ((23, -100), (I64_MAX, -123 + I64_MAX), (-123, -246), (-456, -579)):
        assert pz.decrypt(pk, sk, pz.add_plain(pk, c0, p)) == want
    c0 = enc(pk, I64_MIN)
    assert pz.decrypt(pk, sk, pz.add_plain(pk, c0, I64_MAX)) == -1
    assert pz.decrypt(pk, sk, pz.add_plain(pk, c0, -1)) == I64_MIN - 1


@pytest.mark.parametrize("x", [I64_MIN, -1234, -2, -1, 0, 1, 2, 1234, I64_MAX])
def test_big_number_enc_dec_sub(key1024, x):
    """paillier_test.cc:190-233 (BigNumberTest EncDec / SubTest)."""
    pk, sk = key1024
    c = enc(pk, x, 9)
    assert pz.decrypt(pk, sk, c) == x
    share_a = I64_MAX
    share_b = pz.decrypt(pk, sk, pz.sub_plain(pk, c, share_a))
    assert share_a + share_b == x


def test_numpy_sum_works(key1024):
    """numpy_test.cc:111-120: Sum of 0..899 == 899*900/2."""
    pk, sk = key1024
    rs = pz.r_stream(3, 900, pk.key_size // 2)
    cs = [pz.encrypt(pk, i, r) for i, r in enumerate(rs)]
    assert pz.decrypt(pk, sk, pz.sum_(pk, cs)) == 899 * 900 // 2
    with pytest.raises(pz.PaillierError):
        pz.sum_(pk, [])


def test_numpy_select_sum(key1024):
    """numpy_test.cc:122-165 (SelectSum on a 30x30 matrix of 0..899)."""
    pk, sk = key1024
    vals = [[30 * i + j for j in range(30)] for i in range(2)]
    rs = pz.r_stream(4, 4, pk.key_size // 2)
    cs = [[pz.encrypt(pk, vals[i][j], rs[2 * i + j]) for j in range(2)] for i in range(2)]
    s = pz.sum_(pk, [cs[0][0], cs[0][1], cs[1][0], cs[1][1]])
    assert pz.decrypt(pk, sk, s) == 0 + 1 + 30 + 31


def test_numpy_bin_sum_literal_case(key1024):
    """numpy_test.cc:167-183 (BinSum): rows 2..4 of a 5x2 matrix of 0..9,
    10 features, 5 buckets; element (2, 0) of the result is 4."""
    pk, sk = key1024
    order_map = [[1, 3, 2, 2, 3, 3, 0, 0, 0, 0],
                 [2, 3, 0, 1, 0, 1, 2, 3, 0, 1],
                 [2, 1, 1, 1, 0, 2, 0, 1, 1, 1],
                 [3, 2, 2, 0, 0, 1, 1, 1, 2, 3],
                 [0, 0, 2, 2, 3, 3, 0, 3, 2, 2]]
    m = [[2 * i, 2 * i + 1] for i in range(5)]
    sub = [2, 3, 4]
    rs = pz.r_stream(5, 6, pk.key_size // 2)
    x = [[pz.encrypt(pk, m[i][j], rs[2 * k + j]) for j in range(2)] for k, i in enumerate(sub)]
    om = [order_map[i] for i in sub]
    res = pz.bucket_sum(pk, x, om, 5)
    assert len(res) == 5 * 10 and len(res[0]) == 2
    assert pz.decrypt(pk, sk, res[2][0]) == 4
    # empty bucket holds GetZero (Z-form 1); cumsum variant
    assert res[1][0] == 1
    cres = pz.bucket_sum(pk, x, om, 5, cumsum=True)
    assert pz.decrypt(pk, sk, cres[4][1]) == 5 + 7 + 9


@pytest.mark.parametrize("nkm", [(1, 1, 1), (1, 1, 20), (10, 1, 1), (1, 100, 1), (10, 1, 20), (20, 30, 1),
                                 (1, 100, 3), (2, 3, 4), (10, 30, 20)])
def test_numpy_matmul_shapes(key1024, nkm):
    """matmul_test.cc:21-68: ct x pt matmul equals int64 matmul (x starts at
    10, y at 5, as GenMatrix with start values)."""
    pk, sk = key1024
    n, k, m = nkm
    if n * k * m > 2000:
        pytest.skip("kept short on CPU")
    x = np.arange(10, 10 + n * k, dtype=np.int64).reshape(n, k)
    y = np.arange(5, 5 + k * m, dtype=np.int64).reshape(k, m)
    rs = pz.r_stream(6, n * k, pk.key_size // 2)
    cx = [[pz.encrypt(pk, int(x[i, j]), rs[i * k + j]) for j in range(k)] for i in range(n)]
    out = pz.matmul(pk, cx, y.tolist())
    want = x @ y
    got = [[pz.decrypt(pk, sk, out[i][j]) for j in range(m)] for i in range(n)]
    assert np.array_equal(np.array(got), want)


def test_montgomery_view_roundtrip(key1024):
    pk, _ = key1024
    prg = Prg(3)
    for _ in range(10):
        z = prg.below(pk.n2)
        assert pz.from_mont(pk, pz.to_mont(pk, z)) == z


def test_golden_fixtures_reproduce():
    """The committed fixtures are exactly what the oracle computes."""
    data = json.load(open(os.path.join(HERE, "golden", "paillier_z_kat.json")))
    for c in data["cases"]:
        pk, sk = oracle_key(c["key_bits"], c["seed"])
        assert (pk.n, sk.p, sk.q, pk.h_s) == tuple(int(c[k], 16) for k in ("n", "p", "q", "h_s"))
        ms = [int(v) for v in c["m"]]
        rs = [int(v, 16) for v in c["r"]]
        zs = [pz.encrypt(pk, m, r) for m, r in zip(ms, rs)]
        assert [int(v, 16) for v in c["ct_z"]] == zs
        assert [int(v, 16) for v in c["ct_mont"]] == [pz.to_mont(pk, z) for z in zs]
        assert [pz.decrypt(pk, sk, z) for z in zs] == ms
        ks = [int(v) for v in c["k"]]
        assert [int(v, 16) for v in c["mul"]] == [pz.mul(pk, z, k) for z, k in zip(zs, ks)]
        assert int(c["sum"], 16) == pz.sum_(pk, zs)
        assert [int(v, 16) for v in c["negate"]] == [pz.negate(pk, z) for z in zs]
        nz = len(zs)
        assert [int(v, 16) for v in c["sub_next"]] == [pz.sub(pk, zs[i], zs[(i + 1) % nz]) for i in range(nz)]
        km = [int(v) for v in c["k_more"]]
        assert [int(v, 16) for v in c["mul_more"]] == [pz.mul(pk, zs[i], k) for i, k in enumerate(km)]
        big = [int(v) for v in c["m_big"]]
        assert big[0] == pk.n_half - 1 and big[2] == pk.n_half
        zb = [pz.encrypt(pk, m, int(r, 16)) for m, r in zip(big, c["r_big"])]
        assert [int(v, 16) for v in c["ct_big_z"]] == zb
        assert [pz.decrypt(pk, sk, z) for z in zb] == big
        if "sum_0_899" in c:
            e = c["sum_0_899"]
            rs9 = pz.r_stream(e["r_seed"], 900, pk.key_size // 2)
            s9 = pz.sum_(pk, [pz.encrypt(pk, m, r) for m, r in zip(range(900), rs9)])
            assert int(e["ct_z"], 16) == s9 and pz.decrypt(pk, sk, s9) == 404550
            b = c["bucket_sum"]
            rr = pz.r_stream(b["r_seed"], 24, pk.key_size // 2)
            xz = [[pz.encrypt(pk, b["vals"][i][col], rr[2 * i + col]) for col in range(2)] for i in range(12)]
            for key, cs in (("out_z", False), ("out_cumsum_z", True)):
                got = pz.bucket_sum(pk, xz, b["order_map"], b["buckets"], cumsum=cs)
                assert [[int(v, 16) for v in row] for row in b[key]] == got
            mm = c["matmul"]
            rm = pz.r_stream(mm["r_seed"], 12, pk.key_size // 2)
            xmz = [[pz.encrypt(pk, mm["x"][i][j], rm[4 * i + j]) for j in range(4)] for i in range(3)]
            out = pz.matmul(pk, xmz, mm["y"])
            assert [[int(v, 16) for v in row] for row in mm["out_z"]] == out
            want = [[sum(mm["x"][i][k] * mm["y"][k][j] for k in range(4)) for j in range(2)] for i in range(3)]
            assert [[pz.decrypt(pk, sk, v) for v in row] for row in out] == want


@pytest.mark.parametrize("bits,seed", [(1024, 1), (2048, 0)])
def test_c_restatement_matches_python_oracle(bits, seed):
    from oracle import cref

    pk, sk = oracle_key(bits, seed)
    ck = cref.CKey(bits, pk, sk)
    prg = Prg(8)
    ms = [0, 1, -1, I64_MAX, I64_MIN] + [prg.int64_uniform(-(2 ** 62), 2 ** 62) for _ in range(7)]
    rs = pz.r_stream(12, len(ms), pk.key_size // 2)
    ct = ck.encrypt(np.array(ms), ck.r_array(rs), threads=2)
    zs = [pz.encrypt(pk, m, r) for m, r in zip(ms, rs)]
    assert ck.ints(ct) == [pz.to_mont(pk, z) for z in zs]
    d, ovf = ck.decrypt(ct, threads=2)
    assert d.tolist() == ms and ovf.sum() == 0
    ks = [0, 1, -1, -2, I64_MIN, I64_MAX] + [prg.int64_uniform(I64_MIN, I64_MAX + 1) for _ in range(6)]
    mm = ck.mul(ct, np.array(ks), threads=2)
    assert ck.ints(mm) == [pz.to_mont(pk, pz.mul(pk, z, k)) for z, k in zip(zs, ks)]
    assert ck.ints(ck.sum(ct))[0] == pz.to_mont(pk, pz.sum_(pk, zs))


def test_c_restatement_reductions_match_python_oracle():
    """The C restatement's threaded Sum, FeatureWiseBucketSum and MatMul (the
    timed CPU baseline of the reductions) equal the Python oracle."""
    from oracle import cref

    pk, sk = oracle_key(1024, 1)
    ck = cref.CKey(1024, pk, sk)
    rng = np.random.default_rng(21)
    ms = rng.integers(-1000, 1000, size=48)
    zs = [pz.encrypt(pk, int(m), r) for m, r in zip(ms, pz.r_stream(22, 48, pk.key_size // 2))]
    x = ck.cts([pz.to_mont(pk, z) for z in zs])
    assert ck.ints(ck.sum_mt(x, threads=5))[0] == pz.to_mont(pk, pz.sum_(pk, zs))
    om = rng.integers(0, 6, size=(48, 3)).astype(np.uint8)
    got = [pz.from_mont(pk, v) for v in ck.ints(ck.bucket_sum(x, om, 6, threads=2))]
    assert got == [row[0] for row in pz.bucket_sum(pk, [[z] for z in zs], om.tolist(), 6)]
    y = rng.integers(-50, 50, size=(8, 3))
    y[0, 0], y[1, 1] = 0, -1
    out = ck.matmul(x.reshape(6, 8, -1), y, threads=3)
    cx = [[zs[i * 8 + j] for j in range(8)] for i in range(6)]
    assert [pz.from_mont(pk, v) for v in ck.ints(out.reshape(-1, ck.s))] == \
        [v for row in pz.matmul(pk, cx, y.tolist()) for v in row]


@pytest.mark.parametrize("bits,seed", [(1024, 1), (2048, 0)])
@pytest.mark.parametrize("backend", ["openssl", "gmp", "tommath"])
def test_montgomery_radix_conversion(bits, seed, backend):
    """Ciphertexts move between this engine's radix R = 2^(32 S) and a yacl
    backend's: one Montgomery multiplication by radix_constant each way,
    checked with Python integers (the same constants hg_convert_radix
    computes)."""
    from heu_gb300.engine import backend_radix_bits, radix_constant

    pk, sk = oracle_key(bits, seed)
    n2 = pk.n2
    S = bits // 16
    e = backend_radix_bits(n2.bit_length(), backend)
    if backend in ("openssl", "gmp"):
        assert e == 32 * S  # same radix as this engine for these key sizes
    else:
        assert e == 60 * -(-n2.bit_length() // 60) and e != 32 * S
    r_inv = pow(2 ** (32 * S), -1, n2)

    def mm(x, y):
        return x * y * r_inv % n2

    zs = [pz.encrypt(pk, m, r) for m, r in zip([0, 1, -5, 2 ** 40], pz.r_stream(30, 4, pk.key_size // 2))]
    for z in zs:
        ours = pz.to_mont(pk, z)
        theirs = mm(ours, radix_constant(n2, S, e, True))
        assert theirs == z * pow(2, e, n2) % n2
        assert mm(theirs, radix_constant(n2, S, e, False)) == ours

"""heu.numpy reductions on the engine: FeatureWiseBucketSum and MatMul,
bit-exact against the oracle on small shapes and checked through decryption
at the full config-3 sizes."""

import numpy as np
import pytest

import heu_gb300 as hg
from heu_gb300 import capi
from oracle import paillier_z as pz

pytestmark = pytest.mark.gpu


def enc_matrix(key, pk, vals, seed):
    flat = [int(v) for v in np.asarray(vals).reshape(-1)]
    rs = pz.r_stream(seed, len(flat), pk.key_size // 2)
    zs = [pz.encrypt(pk, m, r) for m, r in zip(flat, rs)]
    ct = key.encrypt(np.array(flat, dtype=np.int64), hg.ints_to_limbs(rs, key.r_limbs))
    return ct, zs


def zform(key, ct):
    return hg.limbs_to_ints(key.from_mont(ct.reshape(-1, key.ct_limbs)))


@pytest.mark.parametrize("cumsum", [False, True])
def test_bucket_sum_matches_oracle(gpu_key, cumsum):
    key, pk, sk = gpu_key(1024, 1)
    rng = np.random.default_rng(3)
    rows, cols, feats, buckets = 300, 2, 5, 7
    vals = rng.integers(-1000, 1000, size=(rows, cols))
    om = rng.integers(0, buckets, size=(rows, feats)).astype(np.uint8)
    om[:, 4] = 3  # one feature with every row in one bucket (others empty)
    ct, zs = enc_matrix(key, pk, vals, 51)
    out = key.bucket_sum(ct.reshape(rows, cols, -1), om, buckets, cumsum=cumsum)
    x = [[zs[i * cols + c] for c in range(cols)] for i in range(rows)]
    exp = pz.bucket_sum(pk, x, om.tolist(), buckets, cumsum=cumsum)
    got = zform(key, out)
    assert got == [v for row in exp for v in row]


def test_bin_sum_literal_case(gpu_key):
    """numpy_test.cc:167-183: rows 2..4 of a 5x2 matrix of 0..9, 10 features,
    5 buckets; result (2, 0) decrypts to 4."""
    key, pk, sk = gpu_key(2048, 0)
    order_map = np.array([[1, 3, 2, 2, 3, 3, 0, 0, 0, 0],
                          [2, 3, 0, 1, 0, 1, 2, 3, 0, 1],
                          [2, 1, 1, 1, 0, 2, 0, 1, 1, 1],
                          [3, 2, 2, 0, 0, 1, 1, 1, 2, 3],
                          [0, 0, 2, 2, 3, 3, 0, 3, 2, 2]], dtype=np.uint8)
    m = np.arange(10).reshape(5, 2)
    sub = [2, 3, 4]
    ct, _ = enc_matrix(key, pk, m[sub], 52)
    out = key.bucket_sum(ct.reshape(3, 2, -1), order_map[sub], 5)
    d, _ = key.decrypt(out.reshape(-1, key.ct_limbs))
    d = d.reshape(50, 2)
    assert d[2, 0] == 4


def test_bucket_sum_rejects_bad_bins(gpu_key):
    key, pk, sk = gpu_key(1024, 1)
    ct, _ = enc_matrix(key, pk, [1, 2, 3], 53)
    om = np.array([[0], [9], [1]], dtype=np.uint8)
    with pytest.raises(hg.HgError) as ei:
        key.bucket_sum(ct, om, 4)
    assert ei.value.code == capi.HG_ERR_INVALID


@pytest.mark.parametrize("nkm", [(1, 1, 1), (1, 1, 20), (10, 1, 1), (1, 100, 1), (10, 1, 20), (20, 30, 1),
                                 (1, 100, 3), (2, 3, 4), (10, 30, 20)])
def test_matmul_shapes_match_oracle(gpu_key, nkm):
    """matmul_test.cc:21-68 shapes (x from 10, y from 5), ct x pt."""
    key, pk, sk = gpu_key(1024, 1)
    n, k, m = nkm
    x = np.arange(10, 10 + n * k, dtype=np.int64).reshape(n, k)
    y = np.arange(5, 5 + k * m, dtype=np.int64).reshape(k, m)
    ct, zs = enc_matrix(key, pk, x, 54)
    out = key.matmul(ct.reshape(n, k, -1), y)
    d, ovf = key.decrypt(out.reshape(-1, key.ct_limbs))
    assert ovf.sum() == 0 and np.array_equal(d.reshape(n, m), x @ y)
    if n * k * m <= 200:
        cx = [[zs[i * k + j] for j in range(k)] for i in range(n)]
        assert zform(key, out) == [v for row in pz.matmul(pk, cx, y.tolist()) for v in row]


def test_matmul_signed_and_extreme_scalars(gpu_key):
    key, pk, sk = gpu_key(2048, 0)
    rng = np.random.default_rng(9)
    x = rng.integers(-(2 ** 20), 2 ** 20, size=(3, 11))
    y = rng.integers(-(2 ** 15), 2 ** 15, size=(11, 4))
    y[0, 0], y[1, 1], y[2, 2] = 0, -1, 2 ** 40
    ct, zs = enc_matrix(key, pk, x, 55)
    out = key.matmul(ct.reshape(3, 11, -1), y)
    cx = [[zs[i * 11 + j] for j in range(11)] for i in range(3)]
    assert zform(key, out) == [v for row in pz.matmul(pk, cx, y.tolist()) for v in row]
    yz = np.zeros((11, 2), dtype=np.int64)
    out = key.matmul(ct.reshape(3, 11, -1), yz)
    assert zform(key, out) == [1] * 6
    yb = np.full((11, 1), -(2 ** 62), dtype=np.int64)
    out = key.matmul(ct.reshape(3, 11, -1), yb)
    assert zform(key, out) == [v for row in pz.matmul(pk, cx, yb.tolist()) for v in row]


def test_matmul_bigint_plaintexts(gpu_key):
    """MatMul with plaintext entries wider than int64 (numpy/evaluator.cc:
    208-353 takes any PMatrix), including negative ones and n/2."""
    key, pk, sk = gpu_key(2048, 0)
    rng = np.random.default_rng(10)
    x = rng.integers(-(2 ** 20), 2 ** 20, size=(2, 5))
    ct, zs = enc_matrix(key, pk, x, 56)
    y = np.array([[2 ** 70, -(2 ** 100), 3], [0, pk.n // 2, -1], [-(pk.n // 2), 5, 2 ** 64],
                  [1, -(2 ** 63), 2 ** 63], [-(2 ** 65) + 3, 7, 0]], dtype=object)
    out = key.matmul(ct.reshape(2, 5, -1), y)
    cx = [[zs[i * 5 + j] for j in range(5)] for i in range(2)]
    assert zform(key, out) == [v for row in pz.matmul(pk, cx, y.tolist()) for v in row]
    # non-negative wide entries take no offset
    yp = np.array([[2 ** 80 + i * j for j in range(3)] for i in range(5)], dtype=object)
    out = key.matmul(ct.reshape(2, 5, -1), yp)
    assert zform(key, out) == [v for row in pz.matmul(pk, cx, yp.tolist()) for v in row]


def test_config3_bucket_sum_full_size(gpu_key):
    """2^20 fixed-point gradients (scale 2^20), 64 features x 256 buckets:
    decrypted bucket sums equal the integer bucket sums."""
    key, pk, sk = gpu_key(2048, 0, 12)
    rows, feats, buckets = 1 << 20, 64, 256
    rng = np.random.default_rng(31)
    g = np.round(rng.standard_normal(rows) * (1 << 20)).astype(np.int64)
    r = rng.integers(0, 2 ** 32, size=(rows, key.r_limbs), dtype=np.uint64).astype(np.uint32)
    ct = key.encrypt(g, r)
    om = rng.integers(0, buckets, size=(rows, feats)).astype(np.uint8)
    out = key.bucket_sum(ct, om, buckets)
    d, ovf = key.decrypt(out.reshape(-1, key.ct_limbs))
    assert ovf.sum() == 0
    exact = np.zeros((feats, buckets), dtype=np.int64)
    for f in range(feats):
        np.add.at(exact[f], om[:, f], g)
    assert np.array_equal(d.reshape(feats, buckets), exact)


def test_config3_matmul_full_size(gpu_key):
    """4096 x 256 ciphertexts @ 256 x 64 int32 in [-2^15, 2^15): decrypted
    result equals the int64 matmul."""
    key, pk, sk = gpu_key(2048, 0, 12)
    M, K, N = 4096, 256, 64
    rng = np.random.default_rng(32)
    x = np.round(rng.standard_normal((M, K)) * (1 << 20)).astype(np.int64)
    y = rng.integers(-(2 ** 15), 2 ** 15, size=(K, N), dtype=np.int64)
    r = rng.integers(0, 2 ** 32, size=(M * K, key.r_limbs), dtype=np.uint64).astype(np.uint32)
    ct = key.encrypt(x.reshape(-1), r)
    out = key.matmul(ct.reshape(M, K, -1), y)
    d, ovf = key.decrypt(out.reshape(-1, key.ct_limbs))
    assert ovf.sum() == 0
    assert np.array_equal(d.reshape(M, N), x @ y)


def test_decrypt_in_range(gpu_key):
    """DecryptInRange (numpy/decryptor.cc:24-47): values within range_bits pass,
    one value with more bits raises with the reference's message."""
    key, pk, sk = gpu_key(1024, 1)
    m = np.array([0, 1, -1, 2 ** 20 - 1, -(2 ** 20 - 1), 12345], dtype=np.int64)
    r = np.zeros((m.size, key.r_limbs), np.uint32)
    r[:, 0] = np.arange(1, m.size + 1)
    ct = key.encrypt(m, r)
    assert np.array_equal(key.decrypt_in_range(ct, 20), m)
    assert key.decrypt_in_range(ct, 200) == m.tolist()
    for bad in (2 ** 20, -(2 ** 20)):
        ct2 = np.concatenate([ct, key.encrypt(np.array([bad]), r[:1])])
        with pytest.raises(ValueError, match="range check failed.*BitCount\\(\\)=21, expected 20"):
            key.decrypt_in_range(ct2, 20)
    big = key.encrypt_bn([pk.n_half], r[:1])
    with pytest.raises(ValueError, match="range check failed"):
        key.decrypt_in_range(big, 63)
    with pytest.raises(ValueError, match="range check failed"):
        key.decrypt_in_range(big, 500)
    assert key.decrypt_in_range(big, pk.n_half.bit_length()) == [pk.n_half]


def test_select_sum_and_batch_select_sum(gpu_key):
    """select_sum / batch_select_sum (numpy/evaluator.h:57-70,
    extension_functions.cc:28-78) against the oracle's Sum of the selection;
    an empty selection equals the engine's own Sub(x00, x00)."""
    key, pk, sk = gpu_key(1024, 1)
    rng = np.random.default_rng(9)
    rows, cols = 40, 3
    vals = rng.integers(-10 ** 6, 10 ** 6, size=(rows, cols))
    ct, zs = enc_matrix(key, pk, vals, 61)
    x = ct.reshape(rows, cols, -1)
    sel = [3, 7, 7, 39]
    got = key.select_sum(x, sel, [0, 2])
    want = pz.sum_(pk, [zs[r * cols + c] for r in sel for c in (0, 2)])
    assert zform(key, got) == [want]
    x1 = x[:, 1]
    got = key.select_sum(x1, slice(5, 25, 2))
    assert zform(key, got) == [pz.sum_(pk, [zs[r * cols + 1] for r in range(5, 25, 2)])]
    zero = key.select_sum(x1, [])
    assert np.array_equal(zero, key.sub(x1[:1], x1[:1]))
    with pytest.raises(ValueError):
        key.select_sum(x1[:0], [])
    sels = [list(rng.integers(0, rows, size=int(rng.integers(0, 6)))) for _ in range(300)]
    sels[5] = []
    outs = key.batch_select_sum(x1, sels)
    assert outs.shape == (300, key.ct_limbs)
    for i in (0, 5, 17, 255, 256, 299):
        want = pz.sum_(pk, [zs[r * cols + 1] for r in sels[i]]) if sels[i] else 1
        assert zform(key, outs[i:i + 1]) == [want], i
    dec, _ = key.decrypt(outs)
    assert dec.tolist() == [int(sum(vals[r, 1] for r in s)) for s in sels]


def test_bucket_sum_equals_select_sum_per_bucket(gpu_key):
    """pylib numpy_test.py:469-560: every bucket of FeatureWiseBucketSum is the
    select_sum of its rows — byte for byte here, since both are the same
    product mod n^2."""
    key, pk, sk = gpu_key(1024, 1)
    rng = np.random.default_rng(21)
    rows, feats, buckets = 120, 3, 6
    vals = rng.integers(-10 ** 6, 10 ** 6, size=rows)
    ct, _ = enc_matrix(key, pk, vals, 71)
    om = rng.integers(0, buckets, size=(rows, feats)).astype(np.uint8)
    out = key.bucket_sum(ct, om, buckets).reshape(feats * buckets, -1)
    for f in range(feats):
        for b in range(buckets):
            sel = np.nonzero(om[:, f] == b)[0]
            assert np.array_equal(out[f * buckets + b], key.select_sum(ct, sel).reshape(-1)), (f, b)
    sels = [np.nonzero(om[:, f] == b)[0] for f in range(feats) for b in range(buckets)]
    assert np.array_equal(key.batch_select_sum(ct, sels), out)

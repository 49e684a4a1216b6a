"""Okamoto-Uchiyama on the engine (hg_ou_keygen / hg_ou_key_load and the
shared C-ABI calls): bit-exact against the OU oracle (oracle/ou.py, which
restates heu/library/algorithms/ou) on the same keys and r stream, at
1024 / 2048 / 3072 bits; Montgomery and Z forms compared."""

import numpy as np
import pytest

import heu_gb300 as hg
import heu_gb300.engine as eng
from heu_gb300 import capi
from oracle import ou
from oracle.prg import Prg

pytestmark = pytest.mark.gpu

I64_MIN, I64_MAX = -(2 ** 63), 2 ** 63 - 1
_OU = {}


@pytest.fixture(scope="module", params=[(1024, 5), (2048, 0), (3072, 7)], ids=lambda p: f"ou{p[0]}")
def oukey(request, gpu_ctx):
    bits, seed = request.param
    if (bits, seed) not in _OU:
        k = eng.ou_keygen(bits, seed)
        pk = ou.PublicKey(k["n"], k["G"], k["H"], 1 << k["max_pt_bits"])
        sk = ou.SecretKey(k["p"], k["q"], k["t"], k["gp_inv"])
        key = gpu_ctx.load_ou_key(bits, k["n"], k["G"], k["H"], k["max_pt_bits"], k["p"], k["q"], k["t"],
                                  k["gp_inv"], table_window=8)
        assert key.ct_limbs == pk.S and key.r_limbs == 4
        _OU[(bits, seed)] = (key, pk, sk)
    return _OU[(bits, seed)]


def rl(key, rs):
    return hg.ints_to_limbs(rs, key.r_limbs)


def ct_eq(key, pk, ct, zs, what):
    assert hg.limbs_to_ints(ct) == [ou.to_mont(pk, z) for z in zs], what + " (Montgomery)"
    assert hg.limbs_to_ints(key.from_mont(ct)) == zs, what + " (Z)"


def mont(key, pk, zs):
    return hg.ints_to_limbs([ou.to_mont(pk, z) for z in zs], key.ct_limbs)


EDGE = [0, 1, -1, 2, -2, -12345, 123, 2 ** 31 - 1, -(2 ** 31), I64_MAX, I64_MIN, 6543212]


def test_encrypt_decrypt_match_oracle(oukey):
    key, pk, sk = oukey
    prg = Prg(11)
    ms = EDGE + [prg.int64_uniform(I64_MIN, I64_MAX + 1) for _ in range(20)]
    rs = [prg.randbits(pk.random_bits) for _ in ms]
    ct = key.encrypt(np.array(ms, dtype=np.int64), rl(key, rs))
    zs = [ou.encrypt(pk, m, r) for m, r in zip(ms, rs)]
    ct_eq(key, pk, ct, zs, "encrypt")
    d, ovf = key.decrypt(ct)
    assert d.tolist() == ms and ovf.sum() == 0
    assert key.decrypt_bn(ct) == ms
    # encrypt_zero / randomize: H^r
    ct_eq(key, pk, key.encrypt_zero(rl(key, rs)), [ou.encrypt_zero(pk, r) for r in rs], "encrypt_zero")
    r2 = [prg.randbits(pk.random_bits) for _ in ms]
    ct_eq(key, pk, key.randomize(ct, rl(key, r2)), [ou.randomize(pk, z, r) for z, r in zip(zs, r2)], "randomize")


def test_full_range_plaintexts(oukey):
    key, pk, sk = oukey
    prg = Prg(12)
    mx = pk.max_plaintext
    ms = [mx, -mx, mx - 1, -(mx - 1), 2 ** 100 + 7, -(2 ** 70), 0, 5]
    rs = [prg.randbits(pk.random_bits) for _ in ms]
    ct = key.encrypt_bn(ms, rl(key, rs))
    ct_eq(key, pk, ct, [ou.encrypt(pk, m, r) for m, r in zip(ms, rs)], "encrypt_bn")
    assert key.decrypt_bn(ct) == ms
    m, ovf = key.decrypt(ct)
    assert ovf.tolist() == [1, 1, 1, 1, 1, 1, 0, 0] and m[6:].tolist() == [0, 5]
    with pytest.raises(hg.HgError) as ei:
        key.encrypt_bn([mx + 1], rl(key, rs[:1]))
    assert ei.value.code == capi.HG_ERR_PT_RANGE


def test_evaluator_matches_oracle(oukey):
    key, pk, sk = oukey
    prg = Prg(13)
    n = len(EDGE)
    ms = [prg.int64_uniform(-(2 ** 40), 2 ** 40) for _ in range(n)]
    rs = [prg.randbits(pk.random_bits) for _ in range(n)]
    zs = [ou.encrypt(pk, m, r) for m, r in zip(ms, rs)]
    a = mont(key, pk, zs)
    b = np.roll(a, 1, axis=0)
    zb = zs[-1:] + zs[:-1]
    ct_eq(key, pk, key.add(a, b), [ou.add(pk, x, y) for x, y in zip(zs, zb)], "add")
    ct_eq(key, pk, key.sub(a, b), [ou.sub(pk, x, y) for x, y in zip(zs, zb)], "sub")
    ct_eq(key, pk, key.negate(a), [ou.negate(pk, x) for x in zs], "negate")
    ks = [0, 1, -1, 2, -2, 2 ** 15 - 1, -(2 ** 15), 2 ** 31 - 1, -(2 ** 31), I64_MAX, I64_MIN, 77]
    ct_eq(key, pk, key.mul(a, np.array(ks, dtype=np.int64)), [ou.mul(pk, z, k) for z, k in zip(zs, ks)], "mul")
    ps = EDGE
    ct_eq(key, pk, key.add_plain(a, np.array(ps, dtype=np.int64)), [ou.add_plain(pk, z, p) for z, p in zip(zs, ps)],
          "add_plain")
    ct_eq(key, pk, key.sub_plain(a, np.array(ps, dtype=np.int64)),
          [ou.add_plain(pk, z, -p) for z, p in zip(zs, ps)], "sub_plain")
    ct_eq(key, pk, key.plain_sub(np.array(ps, dtype=np.int64), a),
          [ou.add_plain(pk, ou.negate(pk, z), p) for z, p in zip(zs, ps)], "plain_sub")
    s = key.sum(a)
    want = 1
    for z in zs:
        want = want * z % pk.n
    ct_eq(key, pk, s, [want], "sum")
    d = key.decrypt_bn(key.mul(key.add(a, b), np.array(ks, dtype=np.int64)))
    assert d == [(x + y) * k for x, y, k in zip(ms, ms[-1:] + ms[:-1], ks)]
    with pytest.raises(hg.HgError) as ei:
        key.add(hg.ints_to_limbs([pk.n], key.ct_limbs), a[:1])
    assert ei.value.code == capi.HG_ERR_CT_RANGE
    with pytest.raises(hg.HgError) as ei:
        key.decrypt(hg.ints_to_limbs([pk.n + 3], key.ct_limbs))
    assert ei.value.code == capi.HG_ERR_CT_RANGE


def test_reductions_and_unsupported_paths(oukey, gpu_ctx):
    key, pk, sk = oukey
    rng = np.random.default_rng(4)
    rows, feats, buckets = 40, 2, 3
    vals = rng.integers(-1000, 1000, size=rows)
    r = np.zeros((rows, key.r_limbs), np.uint32)
    r[:, 0] = np.arange(1, rows + 1)
    ct = key.encrypt(vals, r)
    om = rng.integers(0, buckets, size=(rows, feats)).astype(np.uint8)
    out, _ = key.decrypt(key.bucket_sum(ct, om, buckets).reshape(-1, key.ct_limbs))
    want = np.zeros((feats, buckets), dtype=np.int64)
    for f in range(feats):
        np.add.at(want[f], om[:, f], vals)
    assert np.array_equal(out, want.reshape(-1))
    y = rng.integers(-50, 50, size=(4, 2))
    x = ct[:12].reshape(3, 4, -1)
    mm, _ = key.decrypt(key.matmul(x, y).reshape(-1, key.ct_limbs))
    assert np.array_equal(mm.reshape(3, 2), vals[:12].reshape(3, 4) @ y)
    with pytest.raises(hg.HgError) as ei:
        hg.Server(gpu_ctx).store(key, ct)
    assert ei.value.code == capi.HG_ERR_UNSUPPORTED


def test_full_size_roundtrip_2048(gpu_ctx):
    """2^18 ciphertexts at 2048 bits: Encrypt -> Add -> Decrypt equals int64
    arithmetic (size-independent property)."""
    key, pk, sk = _OU.get((2048, 0)) or (None, None, None)
    if key is None:
        pytest.skip("2048-bit OU key not loaded")
    n = 1 << 18
    rng = np.random.default_rng(8)
    m = rng.integers(-(2 ** 62), 2 ** 62, size=n)
    r = rng.integers(0, 2 ** 32, size=(n, key.r_limbs), dtype=np.uint64).astype(np.uint32)
    r[:, 3] &= (1 << (pk.random_bits - 96)) - 1
    ct = key.encrypt(m, r)
    d, ovf = key.decrypt(key.add(ct, ct))
    assert ovf.sum() == 0 and np.array_equal(d, 2 * m)

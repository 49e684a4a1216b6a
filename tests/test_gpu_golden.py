"""The engine reproduces the committed golden fixtures (tests/golden) byte
for byte at 1024/2048/3072 bits: ciphertexts in Montgomery and Z form,
decryptions, add, sub, negate, signed scalar mul (int32/int64 extremes and
random 64-bit scalars), sum, full-range plaintexts +-(n/2 - 1) and +-n/2,
and (1024 bits) the Sum of 0..899, a bucket-sum with an empty bucket and a
MatMul."""

import json
import os

import numpy as np
import pytest

import heu_gb300 as hg

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = json.load(open(os.path.join(HERE, "golden", "paillier_z_kat.json")))["cases"]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"k{c['key_bits']}")
def test_engine_reproduces_golden(gpu_ctx, case):
    bits = case["key_bits"]
    H = lambda v: int(v, 16)  # noqa: E731
    key = gpu_ctx.load_key(bits, H(case["n"]), H(case["h_s"]), H(case["p"]), H(case["q"]), table_window=9)
    ms = np.array([int(v) for v in case["m"]], dtype=np.int64)
    rs = hg.ints_to_limbs([H(v) for v in case["r"]], key.r_limbs)
    ct = key.encrypt(ms, rs)
    assert hg.limbs_to_ints(ct) == [H(v) for v in case["ct_mont"]]
    assert hg.limbs_to_ints(key.from_mont(ct)) == [H(v) for v in case["ct_z"]]
    d, ovf = key.decrypt(ct)
    assert d.tolist() == ms.tolist() and ovf.sum() == 0
    nxt = np.roll(ct, -1, axis=0)
    assert hg.limbs_to_ints(key.from_mont(key.add(ct, nxt))) == [H(v) for v in case["add_next"]]
    assert hg.limbs_to_ints(key.from_mont(key.negate(ct))) == [H(v) for v in case["negate"]]
    ks = np.array([int(v) for v in case["k"]], dtype=np.int64)
    assert hg.limbs_to_ints(key.from_mont(key.mul(ct, ks))) == [H(v) for v in case["mul"]]
    assert hg.limbs_to_ints(key.from_mont(key.sum(ct))) == [H(case["sum"])]
    assert hg.limbs_to_ints(key.from_mont(key.add_plain(ct, ms))) == [H(v) for v in case["add_plain"]]
    Z = lambda a: hg.limbs_to_ints(key.from_mont(a))  # noqa: E731
    assert Z(key.sub(ct, nxt)) == [H(v) for v in case["sub_next"]]
    km = np.array([int(v) for v in case["k_more"]], dtype=np.int64)
    assert Z(key.mul(ct[: len(km)], km)) == [H(v) for v in case["mul_more"]]
    big = [int(v) for v in case["m_big"]]
    cb = key.encrypt_bn(big, hg.ints_to_limbs([H(v) for v in case["r_big"]], key.r_limbs))
    assert Z(cb) == [H(v) for v in case["ct_big_z"]]
    assert key.decrypt_bn(cb) == big
    if "sum_0_899" in case:
        from oracle import paillier_z as pz

        e = case["sum_0_899"]
        r9 = hg.ints_to_limbs(pz.r_stream(e["r_seed"], 900, bits // 2), key.r_limbs)
        c9 = key.encrypt(np.arange(900, dtype=np.int64), r9)
        s9 = key.sum(c9)
        assert Z(s9) == [H(e["ct_z"])]
        assert key.decrypt(s9)[0].tolist() == [404550]
        b = case["bucket_sum"]
        vals = np.array(b["vals"], dtype=np.int64)
        rb = hg.ints_to_limbs(pz.r_stream(b["r_seed"], 24, bits // 2), key.r_limbs)
        xb = key.encrypt(vals.reshape(-1), rb).reshape(12, 2, -1)
        om = np.array(b["order_map"], dtype=np.uint8)
        for name, cs in (("out_z", False), ("out_cumsum_z", True)):
            got = key.bucket_sum(xb, om, b["buckets"], cumsum=cs)
            assert Z(got.reshape(-1, key.ct_limbs)) == [H(v) for row in b[name] for v in row]
        mm = case["matmul"]
        rm = hg.ints_to_limbs(pz.r_stream(mm["r_seed"], 12, bits // 2), key.r_limbs)
        xm = key.encrypt(np.array(mm["x"], dtype=np.int64).reshape(-1), rm).reshape(3, 4, -1)
        out = key.matmul(xm, np.array(mm["y"], dtype=np.int64))
        assert Z(out.reshape(-1, key.ct_limbs)) == [H(v) for row in mm["out_z"] for v in row]
    key.free()

"""The engine reproduces the committed golden fixtures (tests/golden) byte
for byte: ciphertexts in Montgomery and Z form, decryptions, add, negate,
signed scalar mul and sum."""

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
    key.free()

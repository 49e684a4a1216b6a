"""The C++ SPI adapter (heu_gb300/cpp/paillier_gb300.h) on the GPU: every
vectorized Encryptor / Decryptor / Evaluator call of tests/cpp/spi_test.cpp
runs through the C-ABI, checks its own decryptions, and prints its
ciphertexts, which must equal the oracle's (paillier_z encryptor.cc:36-49,
evaluator.cc) under the same seeded r stream."""

import subprocess

import pytest

from tests.conftest import oracle_key, parse_spi_output, spi_test_binary

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bits", [1024, 2048])
def test_cpp_spi_matches_oracle(bits):
    from oracle import paillier_z as pz

    exe = spi_test_binary()
    res = subprocess.run([exe, "full", str(bits), "3", "17"], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0 and res.stdout.strip().endswith("OK"), res.stdout[-3000:] + res.stderr
    got = parse_spi_output(res.stdout)
    pk, sk = oracle_key(bits, 3)
    assert int(got["n"], 16) == pk.n

    half = pk.n_half
    pts = [0, 1, -1, 123456789, -987654321, 2 ** 63 - 1, -(2 ** 63) + 1, half, -half, half - 12345]
    a = [5, -7, 1000000, 0]
    b = [11, 3, -2000000, -9]
    rs = pz.r_stream(17, len(pts) + len(a) + len(b), bits // 2)
    mont = lambda z: pz.to_mont(pk, z)  # noqa: E731

    enc = [pz.encrypt(pk, m, r) for m, r in zip(pts, rs[: len(pts)])]
    ca = [pz.encrypt(pk, m, r) for m, r in zip(a, rs[len(pts): len(pts) + len(a)])]
    cb = [pz.encrypt(pk, m, r) for m, r in zip(b, rs[len(pts) + len(a):])]
    for i, c in enumerate(enc):
        assert int(got[f"enc[{i}]"], 16) == mont(c), f"enc[{i}]"
    for i in range(len(a)):
        assert int(got[f"ca[{i}]"], 16) == mont(ca[i])
        assert int(got[f"cb[{i}]"], 16) == mont(cb[i])
        assert int(got[f"add_cc[{i}]"], 16) == mont(pz.add(pk, ca[i], cb[i]))
        assert int(got[f"add_cp[{i}]"], 16) == mont(pz.add_plain(pk, ca[i], b[i]))
        assert int(got[f"sub_cc[{i}]"], 16) == mont(pz.sub(pk, ca[i], cb[i]))
        assert int(got[f"mul_cp[{i}]"], 16) == mont(pz.mul(pk, ca[i], b[i]))
        assert int(got[f"neg[{i}]"], 16) == mont(pz.negate(pk, ca[i]))
    assert int(got["sum"], 16) == mont(pz.sum_(pk, ca))
    e60 = int(got["radix60_bits"])
    assert e60 == 60 * -(-pk.n2.bit_length() // 60)
    for i in range(len(a)):
        z = int(got[f"radix60[{i}]"], 16) * pow(2, -e60, pk.n2) % pk.n2
        assert pz.decrypt(pk, sk, z) == a[i], f"radix60[{i}]"
    wide = [half, -half, 1 - half, 2 ** 64]
    for i, kv in enumerate(wide):
        assert int(got[f"mul_big[{i}]"], 16) == mont(pz.mul(pk, ca[i], kv)), f"mul_big[{i}]"
    assert pz.decrypt(pk, sk, pz.from_mont(pk, int(got["sum"], 16))) == sum(a)

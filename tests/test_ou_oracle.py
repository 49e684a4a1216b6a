"""The Okamoto-Uchiyama oracle (oracle/ou.py) pinned against every literal
expectation of the reference's OU tests, and the engine's host key
generation against the oracle (no GPU needed).

  ou_test.cc:27-55    Serialize case: Decrypt(Encrypt(-12345)), Mul by m0 -> m0^2
  ou_test.cc:57-117   CiphertextEvaluate: add, mul by 2, randomize, mul by 1/0/-1/-2
  ou_test.cc:119-142  MinMaxDecrypt: p/2 and bound+1 rejected, +-bound round-trip
  evaluator_test.cc   NegateInplace / CriticalValue over int64 extremes
  key_generator_test.cc: n has at least key_size bits
"""

import pytest

import heu_gb300.engine as eng
from oracle import ou
from oracle.paillier_z import PaillierError
from oracle.prg import Prg

I64_MIN, I64_MAX = -(2 ** 63), 2 ** 63 - 1
_KEYS = {}


def key(bits, seed):
    if (bits, seed) not in _KEYS:
        _KEYS[(bits, seed)] = ou.keygen(bits, seed)
    return _KEYS[(bits, seed)]


def _r(prg, pk):
    return prg.randbits(pk.random_bits)


@pytest.mark.parametrize("bits,seed", [(1024, 5), (2048, 0)])
def test_keygen_invariants(bits, seed):
    pk, sk = key(bits, seed)
    assert pk.n.bit_length() >= bits  # key_generator_test.cc
    assert sk.p * sk.p * sk.q == pk.n
    assert (sk.p - 1) % sk.t == 0  # p = t*u + 1
    assert pk.max_plaintext == 1 << (sk.p_half.bit_length() - 1)
    assert pk.G * pk.G_inv % pk.n == 1


def test_reference_ou_test_expectations():
    pk, sk = key(2048, 0)
    prg = Prg(31)
    m0 = -12345
    ct = ou.encrypt(pk, m0, _r(prg, pk))
    assert ou.decrypt(pk, sk, ct) == m0
    assert ou.decrypt(pk, sk, ou.mul(pk, ct, m0)) == m0 * m0
    ct0 = ou.encrypt(pk, -12345, _r(prg, pk))
    assert ou.decrypt(pk, sk, ou.add(pk, ct0, ct0)) == -12345 * 2
    res = ou.mul(pk, ct0, 2)
    assert ou.decrypt(pk, sk, res) == -12345 * 2
    assert ou.decrypt(pk, sk, ou.randomize(pk, res, _r(prg, pk))) == -12345 * 2
    ct1 = ou.encrypt(pk, 123, _r(prg, pk))
    assert ou.decrypt(pk, sk, ou.add(pk, ct1, ct1)) == 246
    assert ou.decrypt(pk, sk, ou.add(pk, ct0, ct1)) == -12345 + 123
    assert ou.decrypt(pk, sk, ou.mul(pk, ct1, 1)) == 123
    z = ou.mul(pk, ct1, 0)
    assert ou.decrypt(pk, sk, z) == 0
    zr = ou.randomize(pk, z, _r(prg, pk))
    assert zr != 0 and ou.decrypt(pk, sk, zr) == 0
    assert ou.decrypt(pk, sk, ou.mul(pk, ct1, -1)) == -123
    assert ou.decrypt(pk, sk, ou.mul(pk, ct1, -2)) == -246
    # MinMaxDecrypt
    with pytest.raises(PaillierError):
        ou.encrypt(pk, sk.p // 2, 1)
    with pytest.raises(PaillierError):
        ou.encrypt(pk, pk.max_plaintext + 1, 1)
    for m in (pk.max_plaintext, -pk.max_plaintext):
        assert ou.decrypt(pk, sk, ou.encrypt(pk, m, _r(prg, pk))) == m
    with pytest.raises(PaillierError):
        ou.encrypt(pk, -pk.max_plaintext - 1, 1)


@pytest.mark.parametrize("m", [0, 1, -1, 2, -2, 4, -4, 1024, -1024, 100000, -100000, I64_MAX // 2,
                               -(I64_MAX // 2), I64_MAX, I64_MIN])
def test_negate_and_critical_values(m):
    pk, sk = key(1024, 5)
    prg = Prg(abs(m) % 1000 + 3)
    ct = ou.encrypt(pk, m, _r(prg, pk))
    assert ou.decrypt(pk, sk, ou.negate(pk, ct)) == -m
    for k in (0, 1, -1, 2, -2):
        assert ou.decrypt(pk, sk, ou.mul(pk, ct, k)) == m * k


@pytest.mark.parametrize("bits,seed", [(1024, 5), (2048, 0)])
def test_engine_keygen_matches_oracle(bits, seed):
    k = eng.ou_keygen(bits, seed)
    pk, sk = key(bits, seed)
    assert (k["n"], k["G"], k["H"]) == (pk.n, pk.G, pk.H)
    assert (k["p"], k["q"], k["t"], k["gp_inv"]) == (sk.p, sk.q, sk.t, sk.gp_inv)
    assert 1 << k["max_pt_bits"] == pk.max_plaintext

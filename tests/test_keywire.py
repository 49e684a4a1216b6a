"""HEU's key wire format (heu_gb300/keywire.py) on the CPU: the layouts of
paillier_zahlen/public_key.h:60-93, secret_key.h:60-93, ou/public_key.h:134-165
and ou/secret_key.h:37 decode with msgpack-python to the expected fields,
keys round-trip, damaged buffers are rejected, and hnp.setup takes the bytes
(against a stand-in context that records the key load)."""

import struct

import pytest

from heu_gb300 import hnp, keywire
from oracle import ou
from tests.conftest import oracle_key


def _le(v):
    return v.to_bytes((v.bit_length() + 7) // 8, "little")


def test_zpaillier_keys_layout_and_round_trip():
    msgpack = pytest.importorskip("msgpack")
    pk, sk = oracle_key(1024, 1)
    pb = keywire.serialize_public_key({"n": pk.n, "h_s": pk.h_s}, "zpaillier")
    assert pb[-8:] == struct.pack("<Q", 4)
    assert msgpack.unpackb(pb[:-8], raw=True) == [_le(pk.n), _le(pk.h_s)]
    assert keywire.deserialize_public_key(pb) == ("zpaillier", {"n": pk.n, "h_s": pk.h_s})
    sb = keywire.serialize_secret_key({"p": sk.p, "q": sk.q}, pk.n, "zpaillier")
    lam = (sk.p - 1) * (sk.q - 1) // 2
    assert msgpack.unpackb(sb[:-8], raw=True) == [_le(lam), _le(pow(lam, -1, pk.n)), _le(sk.p), _le(sk.q)]
    assert keywire.deserialize_secret_key(sb) == ("zpaillier", {"p": sk.p, "q": sk.q})


def test_ou_keys_layout_and_round_trip():
    msgpack = pytest.importorskip("msgpack")
    opk, osk = ou.keygen(1024, 3)
    mpb = opk.max_plaintext.bit_length() - 1
    d = {"n": opk.n, "G": opk.G, "H": opk.H, "max_pt_bits": mpb}
    pb = keywire.serialize_public_key(d, "ou")
    assert pb[-8:] == struct.pack("<Q", 1)
    assert msgpack.unpackb(pb[:-8], raw=True) == [_le(opk.n), _le(opk.G), _le(opk.H), mpb]
    assert keywire.deserialize_public_key(pb) == ("ou", d)
    s = {"p": osk.p, "q": osk.q, "t": osk.t, "gp_inv": osk.gp_inv}
    sb = keywire.serialize_secret_key(s, opk.n, "ou")
    fields = msgpack.unpackb(sb[:-8], raw=True)
    assert len(fields) == 7 and fields[4] == _le(osk.p * osk.p) and fields[6] == _le(opk.n)
    assert keywire.deserialize_secret_key(sb) == ("ou", dict(s, n=opk.n))


def test_damaged_key_buffers_are_rejected():
    pk, sk = oracle_key(1024, 1)
    pb = keywire.serialize_public_key({"n": pk.n, "h_s": pk.h_s}, "zpaillier")
    sb = keywire.serialize_secret_key({"p": sk.p, "q": sk.q}, pk.n, "zpaillier")
    bad = [pb[:10] + pb[-8:], pb[:-8] + struct.pack("<Q", 9), b"\x93" + pb[1:], pb[:5]]
    for b in bad:
        with pytest.raises(keywire.KeyFormatError):
            keywire.deserialize_public_key(b)
    lam = (sk.p - 1) * (sk.q - 1) // 2
    fields = (lam + 2, pow(lam, -1, pk.n), sk.p, sk.q)  # lambda that does not match p, q
    wrong = keywire._with_schema(keywire._array([keywire._bigint(v) for v in fields]), 4)
    with pytest.raises(keywire.KeyFormatError, match="disagree"):
        keywire.deserialize_secret_key(wrong)
    with pytest.raises(keywire.KeyFormatError):
        keywire.deserialize_secret_key(sb[:-9] + sb[-8:])


def test_setup_from_key_bytes():
    calls = []

    class _Key:
        ct_limbs, r_limbs, pt_limbs = 64, 16, 32

    class _Ctx:
        def load_key(self, bits, n, h_s, p=None, q=None, table_window=0):
            calls.append((bits, n, h_s, p, q))
            return _Key()

    pk, sk = oracle_key(1024, 1)
    pb = keywire.serialize_public_key({"n": pk.n, "h_s": pk.h_s}, "zpaillier")
    sb = keywire.serialize_secret_key({"p": sk.p, "q": sk.q}, pk.n, "zpaillier")
    kit = hnp.setup(pb, context=_Ctx())
    assert calls[-1] == (1024, pk.n, pk.h_s, None, None) and kit.secret_key is None
    assert kit.public_key_bytes() == pb
    kit = hnp.setup(pb, context=_Ctx(), secret_key=sb)
    assert calls[-1] == (1024, pk.n, pk.h_s, sk.p, sk.q) and kit.secret_key == {"p": sk.p, "q": sk.q}
    assert kit.secret_key_bytes() == sb
    other_pk, _ = oracle_key(1024, 2)
    ob = keywire.serialize_public_key({"n": other_pk.n, "h_s": other_pk.h_s}, "zpaillier")
    with pytest.raises(ValueError, match="not paired"):
        hnp.setup(ob, context=_Ctx(), secret_key={"p": sk.p, "q": sk.q, "n": pk.n})

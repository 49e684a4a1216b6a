"""Host logic of the heu.numpy-style layer (no GPU): plaintext conversion
and the broadcasting index maps used by element-wise ops
(numpy/evaluator.cc:160-185 casts shapes the NumPy way)."""

import numpy as np
import pytest

from heu_gb300 import hnp


def test_plaintext_arrays_keep_int64_and_big_values():
    a = hnp.PlaintextArray([[1, 2, 3], [4, 5, 6]])
    assert a.values.dtype == np.int64 and a.shape == (2, 3)
    assert str(a) == "[[1 2 3]\n [4 5 6]]"
    b = hnp.PlaintextArray([2 ** 70, -5])
    assert b.values.dtype == object and b.values.tolist() == [2 ** 70, -5]
    c = hnp.PlaintextArray(np.array([7, -7], dtype=object))
    assert c.values.dtype == np.int64
    assert a[1].to_numpy().tolist() == [4, 5, 6]


def test_broadcast_index_maps():
    shape, ix, iy = hnp._broadcast_index((2, 3), (3,))
    assert shape == (2, 3)
    assert ix.tolist() == [0, 1, 2, 3, 4, 5] and iy.tolist() == [0, 1, 2, 0, 1, 2]
    shape, ix, iy = hnp._broadcast_index((2, 1), (1, 3))
    assert shape == (2, 3) and ix.tolist() == [0, 0, 0, 1, 1, 1] and iy.tolist() == [0, 1, 2, 0, 1, 2]
    shape, ix, iy = hnp._broadcast_index((), (4,))
    assert shape == (4,) and ix.tolist() == [0, 0, 0, 0]
    with pytest.raises(ValueError, match="broadcast"):
        hnp._broadcast_index((2, 3), (2,))


def test_batch_encoder_packs_like_the_reference():
    """DoEncode (batch_encoder.h:128-135): (second << (64 + pad)) | first on the
    64-bit two's-complement patterns; Decode takes slot i's low 64 bits."""
    e = hnp.BatchEncoder(scale=1, padding_bits=32)
    a = np.array([1, -1, 2 ** 62, -(2 ** 63)], dtype=np.int64)
    b = np.array([-5, 7, -(2 ** 40), 2 ** 63 - 1], dtype=np.int64)
    m = e.pack(a, b, 32)
    vals = [int.from_bytes(row.tobytes(), "little") for row in m]
    assert vals == [((int(y) & (2 ** 64 - 1)) << 96) | (int(x) & (2 ** 64 - 1)) for x, y in zip(a, b)]
    assert np.array_equal(e.unpack(m, 0), a) and np.array_equal(e.unpack(m, 1), b)
    # slot-wise sums survive carries into the padding
    s = vals[0] + vals[1]
    mm = np.frombuffer(s.to_bytes(128, "little"), np.uint32).reshape(1, 32)
    assert e.unpack(mm, 0).tolist() == [0] and e.unpack(mm, 1).tolist() == [2]
    e10 = hnp.BatchEncoder(scale=10)
    m10 = e10.pack([3, -4], [-7, 8], 32)
    assert e10.unpack(m10, 0).tolist() == [3, -4] and e10.unpack(m10, 1).tolist() == [-7, 8]
    with pytest.raises(ValueError):
        e.unpack(m, 2)


def test_setup_rejects_unknown_schema():
    with pytest.raises(ValueError, match="schema"):
        hnp.setup(1024, seed=1, schema="elgamal")


def test_ou_randomness_has_exact_bits():
    """OU r is RandomExactBits(random_bits) (ou/encryptor.cc:12-33): the top
    bit set and nothing above it, for 80 / 110 / 128-bit draws."""

    class _Key:
        r_limbs = 4

    class _Kit:
        key = _Key()

    for n_bits, bits in ((1030, 80), (2051, 110), (3077, 128)):
        from heu_gb300 import engine
        assert engine.ou_random_bits(n_bits) == bits
        kit = _Kit()
        kit.random_bits = bits
        r = hnp.Encryptor(kit)._r(64)
        vals = [sum(int(w) << (32 * i) for i, w in enumerate(row)) for row in r]
        assert all(v.bit_length() == bits for v in vals)


def test_plain_encoders_follow_plain_encoder_h():
    """plain_encoder.h:46-74: Encode = value * scale (a double product
    truncated toward zero), Decode = value / scale (C++ integer division for
    IntegerEncoder, a double for FloatEncoder)."""
    fe = hnp.FloatEncoder()
    enc = fe.encode(np.array([1.5, -1.5, 0.1234567, -2.0000009, 0.0]))
    assert enc.dtype == np.int64 and enc.tolist() == [1500000, -1500000, 123456, -2000000, 0]
    assert np.allclose(fe.decode(enc), [1.5, -1.5, 0.123456, -2.0, 0.0])
    ie = hnp.IntegerEncoder(scale=100)
    assert ie.encode([3, -7]).tolist() == [300, -700]
    assert ie.encode(np.array([2.99, -2.99])).tolist() == [299, -299]
    assert ie.decode(np.array([299, -299, 100, -100])).tolist() == [2, -2, 1, -1]
    big = ie.encode([2 ** 62, -(2 ** 62)])
    assert big.dtype == object and big.tolist() == [2 ** 62 * 100, -(2 ** 62) * 100]
    assert ie.decode(big).tolist() == [2 ** 62, -(2 ** 62)]
    a = hnp.PlaintextArray(fe.encode([[0.5, -0.25]]))
    assert a.to_numpy(fe).tolist() == [[0.5, -0.25]]
    with pytest.raises(ValueError):
        hnp.IntegerEncoder(0)


class _FakeKit:
    class key:  # noqa: N801
        ct_limbs = 2
        key_bits = 64


def test_ciphertext_array_transpose_and_setitem_move_limbs():
    limbs = np.arange(12, dtype=np.uint32).reshape(6, 2)  # six "ciphertexts" of two limbs
    x = hnp.CiphertextArray(_FakeKit, limbs, (2, 3))
    t = x.transpose()
    assert t.shape == (3, 2)
    assert t.limbs[:, 0].tolist() == [0, 6, 2, 8, 4, 10]  # element (i, j) of t is (j, i) of x
    with pytest.raises(ValueError):
        hnp.CiphertextArray(_FakeKit, limbs, (6,)).transpose()
    y = hnp.CiphertextArray(_FakeKit, np.full((2, 2), 99, np.uint32), (2,))
    x[1, 1:] = y
    assert x.limbs[:, 0].tolist() == [0, 2, 4, 6, 99, 99]
    x[0] = hnp.CiphertextArray(_FakeKit, np.full((1, 2), 7, np.uint32), ())  # broadcast one ciphertext
    assert x.limbs[:3, 0].tolist() == [7, 7, 7]
    with pytest.raises(TypeError):
        x[0, 0] = 5


def test_encrypt_with_audit_strings():
    """Audit strings as paillier_zahlen/encryptor.cc:50-54 and
    ou/encryptor.cc:110-114 write them (upper-case hex of m, of the
    randomness term and of c), one per element, in the plaintext's shape;
    the engine key is a stand-in that records its inputs."""

    class _Key:
        ct_limbs, r_limbs = 2, 1

        def encrypt(self, m, r):
            out = np.zeros((len(m), 2), np.uint32)
            out[:, 0] = (np.asarray(m) + 1000).astype(np.uint32)
            out[:, 1] = np.asarray(r).reshape(-1)
            return out

        def encrypt_zero(self, r):
            out = np.zeros((r.shape[0], 2), np.uint32)
            out[:, 0] = r[:, 0] * 2
            return out

    class _Kit:
        key = _Key()
        random_bits = None
        max_plaintext = 2 ** 40

    for schema, tag in (("zpaillier", "rn"), ("ou", "hr")):
        kit = _Kit()
        kit.schema = schema
        enc = hnp.Encryptor(kit, r_source=lambda n: np.arange(1, n + 1, dtype=np.uint32).reshape(n, 1))
        ct, audit = enc.encrypt_with_audit(hnp.PlaintextArray([[5, -3]]))
        assert ct.shape == (1, 2) and audit.shape == (1, 2)
        c0 = 1005 + (1 << 32)  # limbs (m + 1000, r) as one integer
        c1 = 997 + (2 << 32)
        assert audit[0, 0] == f"p:5,{tag}:2,c:{c0:X}"
        assert audit[0, 1] == f"p:-3,{tag}:4,c:{c1:X}"


def test_setup_from_public_key_picks_scheme_and_key_size():
    """hnp.setup(public_key): the scheme from the key's fields, the key size
    from key_bits or from n (a k-bit ZPaillier n has k bits, an OU n a few
    more), no secret part; the context is a stand-in that records the load."""
    calls = []

    class _Key:
        ct_limbs, r_limbs, pt_limbs = 32, 16, 16

    class _Ctx:
        def load_key(self, bits, n, h_s, p=None, q=None, table_window=0):
            calls.append(("z", bits, p, q))
            return _Key()

        def load_ou_key(self, bits, n, G, H, max_pt_bits, p=None, q=None, t=None, gp_inv=None, table_window=0):
            calls.append(("ou", bits, max_pt_bits, p))
            return _Key()

    n2048 = (1 << 2047) + 12345
    kit = hnp.setup({"n": n2048, "h_s": 7}, context=_Ctx())
    assert calls[-1] == ("z", 2048, None, None) and kit.schema == "zpaillier" and kit.secret_key is None
    with pytest.raises(ValueError, match="public key"):
        kit.decryptor()
    ou_n = (1 << 2050) + 99  # 2051 bits for a 2048-bit OU key
    kit = hnp.setup({"n": ou_n, "G": 3, "H": 5, "max_pt_bits": 680}, context=_Ctx())
    assert calls[-1] == ("ou", 2048, 680, None) and kit.schema == "ou" and kit.max_plaintext == 1 << 680
    kit = hnp.setup({"n": n2048, "h_s": 7, "key_bits": 2048}, context=_Ctx())
    assert calls[-1][1] == 2048 and kit.public_key["key_bits"] == 2048

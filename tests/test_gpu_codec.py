"""PlainEncoder and BatchEncoder on the device (phe/encoding/plain_encoder.h:
46-74, batch_encoder.h:27-140), fused into the encryption and decryption
kernels: the ciphertexts equal those of the host encoders followed by the
plain encryption (same r), and the decodings equal the host decoders on
the decrypted plaintexts."""

import numpy as np
import pytest

import heu_gb300 as hg
from heu_gb300 import capi, hnp
from oracle import paillier_z as pz

pytestmark = pytest.mark.gpu

I64_MIN, I64_MAX = -(2 ** 63), 2 ** 63 - 1


def _r(key, n, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 2 ** 32, size=(n, key.r_limbs), dtype=np.uint64).astype(np.uint32)


def _host_encrypt(key, ints, r):
    return key.encrypt_bn([int(v) for v in ints], r)


@pytest.mark.parametrize("scale", [1, 10 ** 6, 2 ** 62 - 1])
def test_plain_i64_encode_matches_host_encoder(gpu_key, scale):
    key, pk, sk = gpu_key(2048, 0)
    rng = np.random.default_rng(scale % 1000)
    vals = np.array([0, 1, -1, I64_MAX, I64_MIN, 123456789, -987654321] +
                    list(rng.integers(I64_MIN, I64_MAX, size=57)), dtype=np.int64)
    r = _r(key, vals.size, 1)
    got = key.encrypt_encoded(capi.HG_CODEC_PLAIN_I64, scale, vals, r)
    enc = hnp.IntegerEncoder(scale).encode(vals)
    assert np.array_equal(got, _host_encrypt(key, enc, r))
    # a sample against the definitional oracle
    rs = hg.limbs_to_ints(r[:5])
    assert hg.limbs_to_ints(key.from_mont(got[:5])) == [pz.encrypt(pk, int(v) * scale, rv)
                                                       for v, rv in zip(vals[:5], rs)]
    dec, ovf = key.decrypt_decoded(capi.HG_CODEC_PLAIN_I64, scale, got)
    assert ovf.sum() == 0 and np.array_equal(dec, vals)


def test_plain_f64_encode_and_decode_match_host_encoder(gpu_key):
    key, pk, sk = gpu_key(2048, 0)
    rng = np.random.default_rng(3)
    edge = [0.0, -0.0, 1e-7, -1e-7, 0.5, -0.5, 1.5, -2.5, 2.0 ** 53 + 2, 1e30, -1e30, 1.7e290, -3.3e-300,
            123.456789, -9.87654321e12]
    vals = np.array(edge + list(rng.standard_normal(200) * 1e3), dtype=np.float64)
    for scale in (1, 10 ** 6, 2 ** 40 + 7):
        r = _r(key, vals.size, scale % 97)
        got = key.encrypt_encoded(capi.HG_CODEC_PLAIN_F64, scale, vals, r)
        fe = hnp.FloatEncoder(scale)
        ints = fe.encode(vals)
        assert np.array_equal(got, _host_encrypt(key, ints.reshape(-1), r)), f"scale {scale}"
        dec, ovf = key.decrypt_decoded(capi.HG_CODEC_PLAIN_F64, scale, got)
        want = fe.decode(ints)
        assert ovf.sum() == 0
        assert np.array_equal(dec.view(np.uint64), np.asarray(want, dtype=np.float64).view(np.uint64))
        idec, _ = key.decrypt_decoded(capi.HG_CODEC_PLAIN_I64, scale, got)
        small = np.abs(np.asarray(ints, dtype=object)) < 2 ** 62
        assert all(int(a) == int(b) for a, b, s in zip(idec, hnp.IntegerEncoder(scale).decode(ints), small) if s)
    # non-finite values are rejected; decoding after homomorphic addition
    with pytest.raises(hg.HgError) as ei:
        key.encrypt_encoded(capi.HG_CODEC_PLAIN_F64, 10 ** 6, np.array([1.0, np.inf]), _r(key, 2, 5))
    assert ei.value.code == capi.HG_ERR_PT_RANGE
    a = rng.standard_normal(64)
    b = rng.standard_normal(64)
    ca = key.encrypt_encoded(capi.HG_CODEC_PLAIN_F64, 10 ** 6, a, _r(key, 64, 6))
    cb = key.encrypt_encoded(capi.HG_CODEC_PLAIN_F64, 10 ** 6, b, _r(key, 64, 7))
    s, _ = key.decrypt_decoded(capi.HG_CODEC_PLAIN_F64, 10 ** 6, key.add(ca, cb))
    fe = hnp.FloatEncoder(10 ** 6)
    want = fe.decode(np.asarray(fe.encode(a), dtype=np.int64) + np.asarray(fe.encode(b), dtype=np.int64))
    assert np.array_equal(s, want)


def test_plain_decode_overflow_flags(gpu_key):
    key, pk, sk = gpu_key(2048, 0)
    big = [2 ** 70, -(2 ** 70) - 5, pk.n // 2, 12345]
    ct = key.encrypt_bn(big, _r(key, 4, 8))
    out, ovf = key.decrypt_decoded(capi.HG_CODEC_PLAIN_I64, 1, ct)
    assert ovf.tolist() == [1, 1, 1, 0] and out[3] == 12345
    out, ovf = key.decrypt_decoded(capi.HG_CODEC_PLAIN_I64, 2 ** 10, ct)
    assert ovf.tolist() == [0, 0, 1, 0]
    assert out[0] == 2 ** 60 and out[1] == -((2 ** 70 + 5) // 2 ** 10) and out[3] == 12
    f, ovf = key.decrypt_decoded(capi.HG_CODEC_PLAIN_F64, 3, ct)
    assert ovf.tolist() == [0, 0, 1, 0]
    assert f[0] == float(2 ** 70) / 3 and f[1] == float(-(2 ** 70) - 5) / 3 and np.isinf(f[2])


@pytest.mark.parametrize("padding", [32, 64, 17])
def test_batch_encoder_on_device(gpu_key, padding):
    key, pk, sk = gpu_key(2048, 0)
    rng = np.random.default_rng(padding)
    n = 300
    a = rng.integers(-(2 ** 40), 2 ** 40, size=n)
    b = rng.integers(-(2 ** 40), 2 ** 40, size=n)
    a[:4] = [0, -1, I64_MAX // 7, I64_MIN // 7]
    scale = 7
    r = _r(key, n, 11)
    ct = key.encrypt_encoded(capi.HG_CODEC_BATCH_I64, scale, a, r, values2=b, padding_bits=padding)
    # the packed plaintext, as Python integers (batch_encoder.h:119-126)
    mask = 2 ** 64 - 1
    packed = [(((int(y) * scale) & mask) << (64 + padding)) | ((int(x) * scale) & mask) for x, y in zip(a, b)]
    assert np.array_equal(ct, _host_encrypt(key, packed, r))
    if padding % 32 == 0:
        be = hnp.BatchEncoder(scale, padding)
        mags = be.pack(a, b, key.pt_limbs)
        assert np.array_equal(ct, key.encrypt_bn(hg.limbs_to_ints(mags), r))
    # Add of packed ciphertexts adds the slots; decode per slot: the low 64
    # bits of each slot as int64, / scale with C++ division (batch_encoder.h:
    # 85-103), so a doubled slot wraps like the int64 it is read as
    def slot_sum(vals):
        out = []
        for v in vals:
            w = (2 * int(v) * scale) & mask
            w = w - 2 ** 64 if w >= 2 ** 63 else w
            q = abs(w) // scale
            out.append(-q if w < 0 else q)
        return np.array(out, dtype=np.int64)

    s0, s1, neg = key.decrypt_decoded(capi.HG_CODEC_BATCH_I64, scale, key.add(ct, ct), padding_bits=padding)
    assert neg.sum() == 0
    assert np.array_equal(s0, slot_sum(a)) and np.array_equal(s1, slot_sum(b))
    assert np.array_equal(s0[4:], 2 * a[4:]) and np.array_equal(s1, 2 * b)
    f0, f1, _ = key.decrypt_decoded(capi.HG_CODEC_BATCH_F64, scale, ct, padding_bits=padding)
    assert np.array_equal(f0, (a * scale).astype(np.float64) / scale)
    # double inputs: int64(trunc(x * scale))
    fa = rng.standard_normal(n) * 100
    fb = rng.standard_normal(n) * 100
    cf = key.encrypt_encoded(capi.HG_CODEC_BATCH_F64, 1000, fa, r, values2=fb, padding_bits=padding)
    pf = [(((int(np.trunc(y * 1000.0))) & mask) << (64 + padding)) | (int(np.trunc(x * 1000.0)) & mask)
          for x, y in zip(fa, fb)]
    assert np.array_equal(cf, _host_encrypt(key, pf, r))


def test_hnp_encrypt_and_decode_run_on_the_device(gpu_ctx):
    """hnp.Encryptor.encrypt(kit.array(floats, fe)) takes the device codec
    (no host encode pass: the array's encoded values are never computed),
    and gives the ciphertexts of the host path under the same r."""
    kit = hnp.setup(1024, seed=5, context=gpu_ctx, table_window=8)
    fe = kit.float_encoder(10 ** 6)
    rng = np.random.default_rng(12)
    vals = rng.standard_normal((16, 4)) * 1e4
    rsrc = lambda count: _r(kit.key, count, 99)  # noqa: E731
    arr = kit.array(vals, fe)
    ct = kit.encryptor(r_source=rsrc).encrypt(arr)
    assert arr._values is None, "the values were encoded on the host"
    host = kit.encryptor(r_source=rsrc).encrypt(hnp.PlaintextArray(fe.encode(vals)))
    assert np.array_equal(ct.limbs, host.limbs)
    dec = kit.decryptor().decrypt(ct)
    got = dec.to_numpy(fe)
    assert dec._values is None, "decoded through the host path"
    assert np.array_equal(got, fe.decode(fe.encode(vals)))
    be = kit.batch_encoder(scale=1, padding_bits=32)
    a = rng.integers(-1000, 1000, size=10)
    b = rng.integers(-1000, 1000, size=10)
    cb = kit.encryptor().encrypt_batch(a, b, be)
    x, y = kit.decryptor().decrypt_batch(cb, be)
    assert np.array_equal(x, a) and np.array_equal(y, b)

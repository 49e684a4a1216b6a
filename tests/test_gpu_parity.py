"""Bit-exact parity of the sm_103a engine (through the C-ABI) with the
paillier_z oracle on the same keys and the same injected r stream.

Ciphertexts leave the engine in Montgomery form (HEU's representation); each
test checks both that form (c*R mod n^2) and the canonical Z-form.
"""

import numpy as np
import pytest

import heu_gb300 as hg
from heu_gb300 import capi
from oracle import paillier_z as pz
from oracle.prg import Prg

pytestmark = pytest.mark.gpu

KEYS = [(1024, 1), (2048, 0), (3072, 2)]
I64_MIN, I64_MAX = -(2 ** 63), 2 ** 63 - 1
EDGE_M = [0, 1, -1, 2, -2, 12345, -12345, 123, -123, 2 ** 31 - 1, -(2 ** 31), I64_MAX, I64_MIN, 6543212, -456]


def rand_i64(prg, n, lo=I64_MIN, hi=I64_MAX + 1):
    return [prg.int64_uniform(lo, hi) for _ in range(n)]


def r_limbs(pk, rs, key):
    return hg.ints_to_limbs(rs, key.r_limbs)


def to_mont_limbs(pk, key, zs):
    return hg.ints_to_limbs([pz.to_mont(pk, z) for z in zs], key.ct_limbs)


def z_of(key, ct):
    return hg.limbs_to_ints(key.from_mont(ct))


def assert_ct_equal(pk, key, ct, expected_z, what):
    got_m = hg.limbs_to_ints(ct)
    exp_m = [pz.to_mont(pk, z) for z in expected_z]
    bad = [i for i, (a, b) in enumerate(zip(got_m, exp_m)) if a != b]
    assert not bad, f"{what}: {len(bad)} Montgomery-form mismatches, first at {bad[0]}"
    got_z = z_of(key, ct)
    bad = [i for i, (a, b) in enumerate(zip(got_z, expected_z)) if a != b]
    assert not bad, f"{what}: {len(bad)} Z-form mismatches, first at {bad[0]}"


@pytest.fixture(params=KEYS, ids=lambda k: f"k{k[0]}")
def kk(request, gpu_key):
    bits, seed = request.param
    return gpu_key(bits, seed)


def test_encrypt_matches_oracle(kk):
    key, pk, sk = kk
    prg = Prg(11)
    ms = EDGE_M + rand_i64(prg, 49)
    rs = pz.r_stream(7, len(ms), pk.key_size // 2)
    ct = key.encrypt(np.array(ms, dtype=np.int64), r_limbs(pk, rs, key))
    exp = [pz.encrypt(pk, m, r) for m, r in zip(ms, rs)]
    assert_ct_equal(pk, key, ct, exp, "encrypt")


def test_encrypt_edge_randomness(kk):
    key, pk, sk = kk
    top = (1 << (pk.key_size // 2)) - 1
    rs = [0, 1, 2, top, top - 1, 1 << (pk.key_size // 2 - 1), 0x5555 << 100]
    ms = [5] * len(rs)
    ct = key.encrypt(np.array(ms, dtype=np.int64), r_limbs(pk, rs, key))
    assert_ct_equal(pk, key, ct, [pz.encrypt(pk, m, r) for m, r in zip(ms, rs)], "encrypt edge r")


def test_encrypt_zero_and_randomize(kk):
    key, pk, sk = kk
    rs = pz.r_stream(3, 9, pk.key_size // 2)
    ez = key.encrypt_zero(r_limbs(pk, rs, key))
    assert_ct_equal(pk, key, ez, [pz.encrypt_zero(pk, r) for r in rs], "encrypt_zero")
    ms = list(range(-4, 5))
    base_r = pz.r_stream(4, 9, pk.key_size // 2)
    ct = key.encrypt(np.array(ms, dtype=np.int64), r_limbs(pk, base_r, key))
    rr = key.randomize(ct, r_limbs(pk, rs, key))
    exp = [pz.randomize(pk, pz.encrypt(pk, m, r0), r) for m, r0, r in zip(ms, base_r, rs)]
    assert_ct_equal(pk, key, rr, exp, "randomize")


def test_encrypt_bn_bounds(kk):
    key, pk, sk = kk
    nh = pk.n_half
    ms = [nh, -nh, nh - 1, -(nh - 1), 2 ** 64 + 3, -(2 ** 100)]
    rs = pz.r_stream(5, len(ms), pk.key_size // 2)
    ct = key.encrypt_bn(ms, r_limbs(pk, rs, key))
    assert_ct_equal(pk, key, ct, [pz.encrypt(pk, m, r) for m, r in zip(ms, rs)], "encrypt_bn")
    assert key.decrypt_bn(ct) == ms
    # paillier_test.cc:99-119: |m| = n/2 + 1 and n are rejected
    for bad in (nh + 1, -(nh + 1), pk.n - 1):
        with pytest.raises(hg.HgError) as ei:
            key.encrypt_bn([bad], r_limbs(pk, rs[:1], key))
        assert ei.value.code == capi.HG_ERR_PT_RANGE


def test_decrypt_matches_oracle(kk):
    key, pk, sk = kk
    prg = Prg(12)
    ms = EDGE_M + rand_i64(prg, 33)
    rs = pz.r_stream(8, len(ms), pk.key_size // 2)
    zs = [pz.encrypt(pk, m, r) for m, r in zip(ms, rs)]
    ct = to_mont_limbs(pk, key, zs)
    m, ovf = key.decrypt(ct)
    assert ovf.sum() == 0
    assert m.tolist() == ms
    # big plaintexts through the bignum output
    big = [pk.n_half, -pk.n_half, 2 ** 200 + 5, -(2 ** 77)]
    rb = pz.r_stream(9, len(big), pk.key_size // 2)
    ct = to_mont_limbs(pk, key, [pz.encrypt(pk, v, r) for v, r in zip(big, rb)])
    assert key.decrypt_bn(ct) == big
    m, ovf = key.decrypt(ct)
    assert ovf.tolist() == [1, 1, 1, 1]


def test_decrypt_arbitrary_residues(kk):
    """Decrypt of residues that are not fresh encryptions (any c < n^2)."""
    key, pk, sk = kk
    prg = Prg(99)
    zs = [prg.below(pk.n2) for _ in range(20)] + [1, pk.n2 - 1]
    ct = to_mont_limbs(pk, key, zs)
    got = key.decrypt_bn(ct)
    assert got == [pz.decrypt(pk, sk, z) for z in zs]


def test_add_sub_negate(kk):
    key, pk, sk = kk
    prg = Prg(13)
    n = 40
    ma = EDGE_M[:10] + rand_i64(prg, n - 10, -(2 ** 62), 2 ** 62)
    mb = rand_i64(prg, n, -(2 ** 62), 2 ** 62)
    ra = pz.r_stream(21, n, pk.key_size // 2)
    rb = pz.r_stream(22, n, pk.key_size // 2)
    za = [pz.encrypt(pk, m, r) for m, r in zip(ma, ra)]
    zb = [pz.encrypt(pk, m, r) for m, r in zip(mb, rb)]
    ca, cb = to_mont_limbs(pk, key, za), to_mont_limbs(pk, key, zb)
    assert_ct_equal(pk, key, key.add(ca, cb), [pz.add(pk, a, b) for a, b in zip(za, zb)], "add")
    assert_ct_equal(pk, key, key.negate(ca), [pz.negate(pk, a) for a in za], "negate")
    assert_ct_equal(pk, key, key.sub(ca, cb), [pz.sub(pk, a, b) for a, b in zip(za, zb)], "sub")
    m, _ = key.decrypt(key.sub(ca, cb))
    assert m.tolist() == [a - b for a, b in zip(ma, mb)]


def test_add_plain_variants(kk):
    key, pk, sk = kk
    prg = Prg(14)
    ps = EDGE_M + rand_i64(prg, 17)
    n = len(ps)
    ms = rand_i64(prg, n, -(2 ** 40), 2 ** 40)
    rs = pz.r_stream(23, n, pk.key_size // 2)
    zs = [pz.encrypt(pk, m, r) for m, r in zip(ms, rs)]
    c = to_mont_limbs(pk, key, zs)
    p = np.array(ps, dtype=np.int64)
    assert_ct_equal(pk, key, key.add_plain(c, p), [pz.add_plain(pk, z, q) for z, q in zip(zs, ps)], "add_plain")
    assert_ct_equal(pk, key, key.sub_plain(c, p), [pz.sub_plain(pk, z, q) for z, q in zip(zs, ps)], "sub_plain")
    assert_ct_equal(pk, key, key.plain_sub(p, c), [pz.sub_plain_ct(pk, q, z) for z, q in zip(zs, ps)],
                    "plain_sub")


def test_mul_scalars(kk):
    key, pk, sk = kk
    prg = Prg(15)
    ks = [0, 1, -1, 2, -2, 3, -3, 2 ** 15 - 1, -(2 ** 15), 2 ** 31 - 1, -(2 ** 31), I64_MAX, I64_MIN,
          I64_MIN + 1] + rand_i64(prg, 26)
    n = len(ks)
    ms = rand_i64(prg, n, -(2 ** 31), 2 ** 31)
    rs = pz.r_stream(24, n, pk.key_size // 2)
    zs = [pz.encrypt(pk, m, r) for m, r in zip(ms, rs)]
    c = to_mont_limbs(pk, key, zs)
    out = key.mul(c, np.array(ks, dtype=np.int64))
    assert_ct_equal(pk, key, out, [pz.mul(pk, z, k) for z, k in zip(zs, ks)], "mul")


def test_mul_all_positive_skips_inverse(kk):
    key, pk, sk = kk
    ks = [5, 7, 2 ** 40 + 1, 1, 0]
    zs = [pz.encrypt(pk, m, r) for m, r in zip([3, -4, 5, 6, 7], pz.r_stream(25, 5, pk.key_size // 2))]
    out = key.mul(to_mont_limbs(pk, key, zs), np.array(ks, dtype=np.int64))
    assert_ct_equal(pk, key, out, [pz.mul(pk, z, k) for z, k in zip(zs, ks)], "mul positive")


def test_mul_bigint_scalars(kk):
    """Mul(ct, BigInt) (evaluator.cc:99-123): scalars wider than int64, up to
    the width of n^2, byte-equal to the oracle; int64-range values through the
    multi-limb path equal hg_mul's."""
    key, pk, sk = kk
    half = pk.n // 2
    ks = [2 ** 64, -(2 ** 64), 2 ** 200 + 12345, -(2 ** 200), half, -half, half - 1, pk.n, pk.n2 - 1,
          -(pk.n2 - 1), 2 ** 63, -(2 ** 63) - 1, 0, 1, -1, 7]
    prg = Prg(19)
    ks += [prg.below(pk.n) - pk.n // 2 for _ in range(16)]
    n = len(ks)
    ms = rand_i64(prg, n, -(2 ** 31), 2 ** 31)
    zs = [pz.encrypt(pk, m, r) for m, r in zip(ms, pz.r_stream(26, n, pk.key_size // 2))]
    c = to_mont_limbs(pk, key, zs)
    out = key.mul(c, np.array(ks, dtype=object))
    assert_ct_equal(pk, key, out, [pz.mul(pk, z, k) for z, k in zip(zs, ks)], "mul bigint")
    small = [0, 1, -1, 2, -3, I64_MAX, I64_MIN + 1, 2 ** 40]
    assert np.array_equal(key.mul_bn(c[:8], small), key.mul(c[:8], np.array(small, dtype=np.int64)))
    # decryptions: m * k mod n, centred
    dm = key.decrypt_bn(out[:6])
    for got, m, k in zip(dm, ms, ks):
        want = (m * k) % pk.n
        assert got == (want - pk.n if want > pk.n // 2 else want)


def test_mul_bigint_device_form_and_limits(kk):
    torch = pytest.importorskip("torch")
    import ctypes

    key, pk, sk = kk
    ks = [2 ** 100 + 1, -(2 ** 90), 5, 0, -(pk.n // 2)]
    zs = [pz.encrypt(pk, m, r) for m, r in zip([3, -4, 5, 6, 7], pz.r_stream(27, 5, pk.key_size // 2))]
    c = to_mont_limbs(pk, key, zs)
    width = key.ct_limbs // 2
    mags = hg.ints_to_limbs([abs(k) for k in ks], width)
    neg = np.array([k < 0 for k in ks], dtype=np.uint8)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    dc = torch.from_numpy(c.view(np.int32)).cuda()
    dm = torch.from_numpy(mags.view(np.int32)).cuda()
    dn = torch.from_numpy(neg).cuda()
    dout = torch.zeros_like(dc)
    torch.cuda.synchronize()  # the engine's stream does not wait for torch's
    capi.check(key.lib.hg_dev_mul_bn(key.ctx.handle, key.id, P(dc), P(dm), P(dn), width, P(dout), 5, None))
    torch.cuda.synchronize()
    capi.check(key.lib.hg_dev_check(key.ctx.handle))
    got = dout.cpu().numpy().view(np.uint32)
    assert_ct_equal(pk, key, got, [pz.mul(pk, z, k) for z, k in zip(zs, ks)], "dev mul bigint")
    # scalars wider than n^2 are rejected before any work
    too = hg.ints_to_limbs([1], key.ct_limbs + 1)
    out = np.zeros_like(c[:1])
    rc = key.lib.hg_mul_bn(key.ctx.handle, key.id, hg.engine._ptr(c[:1]), hg.engine._ptr(too),
                           hg.engine._ptr(np.zeros(1, np.uint8)), key.ct_limbs + 1, hg.engine._ptr(out), 1)
    assert rc == capi.HG_ERR_INVALID


@pytest.mark.parametrize("count", [1, 2, 3, 17, 255, 256, 257, 900])
def test_sum_counts(gpu_key, count):
    key, pk, sk = gpu_key(2048, 0)
    ms = list(range(count))
    rs = pz.r_stream(30 + count, count, pk.key_size // 2)
    zs = [pz.encrypt(pk, m, r) for m, r in zip(ms, rs)]
    out = key.sum(to_mont_limbs(pk, key, zs))
    assert_ct_equal(pk, key, out, [pz.sum_(pk, zs)], f"sum[{count}]")
    # numpy_test.cc:111-120 (Sum of 0..899)
    m, _ = key.decrypt(out)
    assert int(m[0]) == count * (count - 1) // 2


def test_ciphertext_range_rejected(kk):
    key, pk, sk = kk
    bad = hg.ints_to_limbs([pk.n2, pk.n2 + 5], key.ct_limbs)
    good = to_mont_limbs(pk, key, [pz.encrypt(pk, 1, 1), pz.encrypt(pk, 2, 2)])
    for fn in (lambda: key.add(bad, good), lambda: key.decrypt(bad), lambda: key.mul(bad, [2, 3]),
               lambda: key.negate(bad), lambda: key.sum(bad)):
        with pytest.raises(hg.HgError) as ei:
            fn()
        assert ei.value.code == capi.HG_ERR_CT_RANGE


def test_latency_and_throughput_layouts_agree(gpu_key):
    """Small batches run in the latency layout (a warp per ciphertext mod n^2,
    a half warp per CRT side) and large ones in the throughput layout; both
    give paillier_z's bytes (C restatement) for Encrypt, Mul and Decrypt."""
    import os

    from oracle import cref

    key, pk, sk = gpu_key(2048, 0)
    n = 12288  # above one wave of the latency layout
    rng = np.random.default_rng(41)
    m = rng.integers(-(2 ** 40), 2 ** 40, size=n, dtype=np.int64)
    r = rng.integers(0, 2 ** 32, size=(n, key.r_limbs), dtype=np.uint64).astype(np.uint32)
    k = rng.integers(-(2 ** 63), 2 ** 63 - 1, size=n, dtype=np.int64)
    ck = cref.CKey(2048, pk, sk, window=10)
    threads = os.cpu_count() or 1
    want = ck.encrypt(m, np.ascontiguousarray(r).view(np.uint64), threads).view(np.uint32).reshape(n, -1)
    big = key.encrypt(m, r)
    for small_n in (1, 3, 64, 1000):
        small = key.encrypt(m[:small_n], r[:small_n])
        assert np.array_equal(small, want[:small_n]), f"latency-layout encrypt differs at n={small_n}"
    assert np.array_equal(big, want), "throughput-layout encrypt differs"
    want_mul = ck.mul(np.ascontiguousarray(want).view(np.uint64), k, threads).view(np.uint32).reshape(n, -1)
    assert np.array_equal(key.mul(big[:37], k[:37]), want_mul[:37])
    assert np.array_equal(key.mul(big, k), want_mul)
    d_small, _ = key.decrypt(big[:29])
    d_big, ovf = key.decrypt(big)
    assert np.array_equal(d_small, m[:29]) and np.array_equal(d_big, m) and ovf.sum() == 0


def test_sum_checks_every_input(gpu_key):
    """A value >= n^2 anywhere in a Sum input is rejected (evaluator.cc:21-23
    VALIDATE), not only at the first element of a reduction chunk."""
    key, pk, sk = gpu_key(2048, 0)
    good = pz.to_mont(pk, pz.encrypt(pk, 7, 3))
    for n, bad_at in ((2, 1), (64, 63), (300_000, 12_345), (300_000, 299_999)):
        zs = np.tile(hg.ints_to_limbs([good], key.ct_limbs), (n, 1))
        zs[bad_at] = hg.ints_to_limbs([pk.n2 + 1], key.ct_limbs)[0]
        with pytest.raises(hg.HgError) as ei:
            key.sum(zs)
        assert ei.value.code == capi.HG_ERR_CT_RANGE, (n, bad_at)
    # the device-pointer form reports the same
    torch = pytest.importorskip("torch")
    import ctypes

    zs = np.tile(hg.ints_to_limbs([good], key.ct_limbs), (64, 1))
    zs[63] = hg.ints_to_limbs([pk.n2], key.ct_limbs)[0]
    d = torch.from_numpy(zs.view(np.int32)).cuda()
    out = torch.zeros((1, key.ct_limbs), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()  # the engine's stream does not wait for torch's
    capi.check(key.lib.hg_dev_sum(key.ctx.handle, key.id, ctypes.c_void_p(d.data_ptr()), 64,
                                  ctypes.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    assert key.lib.hg_dev_check(key.ctx.handle) == capi.HG_ERR_CT_RANGE
    # and a valid input still sums after the error
    zs[63] = zs[0]
    assert hg.limbs_to_ints(key.from_mont(key.sum(zs))) == [pz.sum_(pk, [pz.encrypt(pk, 7, 3)] * 64)]


def test_montgomery_conversion_roundtrip(kk):
    key, pk, sk = kk
    prg = Prg(16)
    zs = [prg.below(pk.n2) for _ in range(16)] + [0, 1, pk.n2 - 1]
    zl = hg.ints_to_limbs(zs, key.ct_limbs)
    mont = key.to_mont(zl)
    assert hg.limbs_to_ints(mont) == [pz.to_mont(pk, z) for z in zs]
    assert hg.limbs_to_ints(key.from_mont(mont)) == zs


@pytest.mark.parametrize("backend", ["openssl", "tommath"])
def test_backend_radix_conversion(kk, backend):
    """hg_convert_radix: c * R <-> c * R_ext for a yacl backend's radix."""
    from heu_gb300.engine import backend_radix_bits

    key, pk, sk = kk
    e = backend_radix_bits(pk.n2.bit_length(), backend)
    zs = [pz.encrypt(pk, m, r) for m, r in zip([0, 7, -9, 2 ** 50], pz.r_stream(31, 4, pk.key_size // 2))]
    ours = to_mont_limbs(pk, key, zs)
    ext = key.convert_radix(ours, e, True)
    assert hg.limbs_to_ints(ext) == [z * pow(2, e, pk.n2) % pk.n2 for z in zs]
    assert np.array_equal(key.convert_radix(ext, e, False), ours)


def test_table_window_does_not_change_results(gpu_ctx):
    pk, sk = pz.keygen(1024, 1)
    ms = [1, -2, 3, 2 ** 40]
    rs = pz.r_stream(40, 4, pk.key_size // 2)
    exp = [pz.encrypt(pk, m, r) for m, r in zip(ms, rs)]
    for w in (1, 5, 10, 13):
        key = gpu_ctx.load_key(1024, pk.n, pk.h_s, table_window=w)
        ct = key.encrypt(np.array(ms, dtype=np.int64), hg.ints_to_limbs(rs, key.r_limbs))
        assert_ct_equal(pk, key, ct, exp, f"window {w}")
        with pytest.raises(hg.HgError) as ei:
            key.decrypt(ct)
        assert ei.value.code == capi.HG_ERR_NO_SECRET
        key.free()


def test_engine_keygen_matches_oracle_and_loads(gpu_ctx):
    k = hg.keygen(2048, 0)
    pk, sk = pz.keygen(2048, 0)
    assert (k["n"], k["p"], k["q"], k["h_s"]) == (pk.n, sk.p, sk.q, pk.h_s)


def test_config2_roundtrip_full_size(gpu_key):
    """1,048,576 int64 plaintexts in [-2^40, 2^40): Encrypt -> Decrypt == m,
    Add and Mul checked through decryption (size-independent properties)."""
    key, pk, sk = gpu_key(2048, 0, 12)
    n = 1 << 20
    rng = np.random.default_rng(2)
    m = rng.integers(-(2 ** 40), 2 ** 40, size=n, dtype=np.int64)
    r = rng.integers(0, 2 ** 32, size=(n, key.r_limbs), dtype=np.uint64).astype(np.uint32)
    ct = key.encrypt(m, r)
    dm, ovf = key.decrypt(ct)
    assert ovf.sum() == 0
    assert np.array_equal(dm, m)
    # a few spot checks against the oracle
    for i in (0, 1, n // 2, n - 1):
        rv = hg.limbs_to_ints(r[i:i + 1])[0]
        assert hg.limbs_to_ints(key.from_mont(ct[i:i + 1]))[0] == pz.encrypt(pk, int(m[i]), rv)
    s = key.add(ct, ct[::-1].copy())
    dm, _ = key.decrypt(s)
    assert np.array_equal(dm, m + m[::-1])
    k = rng.integers(-(2 ** 15), 2 ** 15, size=n, dtype=np.int64)
    mm = key.mul(ct, k)
    dm, ovf = key.decrypt(mm)
    assert ovf.sum() == 0
    assert np.array_equal(dm, m * k)


def test_config1_workflow_bit_exact_against_c_restatement(gpu_key):
    """The 10,000-element workflow: 2048-bit key from seed 0, int64 m in
    [-2^31, 2^31), Encrypt, pairwise Add (ct_i + ct_(i+1)), Mul by int32
    k in [-2^15, 2^15), Decrypt.  Every ciphertext is compared byte for byte
    with the C restatement of paillier_z on the same r stream (all elements,
    not a sample), and the decryptions with exact int64 arithmetic."""
    import os

    from oracle import cref

    key, pk, sk = gpu_key(2048, 0, 12)
    n = 10_000
    prg = Prg(1)
    m = np.array([prg.int64_uniform(-(2 ** 31), 2 ** 31) for _ in range(n)], dtype=np.int64)
    k = np.array([prg.int64_uniform(-(2 ** 15), 2 ** 15) for _ in range(n)], dtype=np.int64)
    rs = pz.r_stream(1, n, pk.key_size // 2)
    ck = cref.CKey(2048, pk, sk)
    th = os.cpu_count() or 1

    ct = key.encrypt(m, r_limbs(pk, rs, key))
    ct_c = ck.encrypt(m, ck.r_array(rs), threads=th)
    assert np.array_equal(ct.view(np.uint64), ct_c), "encrypt"

    nxt = np.roll(np.arange(n), -1)
    s = key.add(ct, ct[nxt].copy())
    s_c = ck.add(ct_c, np.ascontiguousarray(ct_c[nxt]), threads=th)
    assert np.array_equal(s.view(np.uint64), s_c), "pairwise add"

    p = key.mul(s, k)
    p_c = ck.mul(s_c, k, threads=th)
    assert np.array_equal(p.view(np.uint64), p_c), "mul"

    d, ovf = key.decrypt(p)
    assert ovf.sum() == 0
    assert np.array_equal(d, (m + m[nxt]) * k)
    d_c, _ = ck.decrypt(p_c[:256], threads=th)
    assert np.array_equal(d[:256], d_c)


def test_empty_batches_and_ragged_tails(kk):
    """count = 0 is a no-op for every element-wise call; Sum of nothing is an
    error as in numpy/evaluator.cc (you cannot sum an empty tensor); batch
    sizes that leave partial warps and partial groups match the oracle."""
    key, pk, sk = kk
    S, RL = key.ct_limbs, key.r_limbs
    e_ct = np.zeros((0, S), np.uint32)
    assert key.encrypt(np.zeros(0, np.int64), np.zeros((0, RL), np.uint32)).shape == (0, S)
    m, ovf = key.decrypt(e_ct)
    assert m.shape == (0,) and ovf.shape == (0,)
    assert key.add(e_ct, e_ct).shape == (0, S)
    assert key.sub(e_ct, e_ct).shape == (0, S)
    assert key.mul(e_ct, np.zeros(0, np.int64)).shape == (0, S)
    assert key.negate(e_ct).shape == (0, S)
    assert key.add_plain(e_ct, np.zeros(0, np.int64)).shape == (0, S)
    with pytest.raises(hg.HgError):
        key.sum(e_ct)
    prg = Prg(77)
    for count in (1, 3, 5, 33, 65):
        ms = rand_i64(prg, count, -(2 ** 50), 2 ** 50)
        ks = rand_i64(prg, count)
        rs = pz.r_stream(700 + count, count, pk.key_size // 2)
        zs = [pz.encrypt(pk, m, r) for m, r in zip(ms, rs)]
        ct = key.encrypt(np.array(ms, dtype=np.int64), r_limbs(pk, rs, key))
        assert_ct_equal(pk, key, ct, zs, f"encrypt[{count}]")
        d, ovf = key.decrypt(ct)
        assert d.tolist() == ms and ovf.sum() == 0
        assert_ct_equal(pk, key, key.mul(ct, np.array(ks, dtype=np.int64)),
                        [pz.mul(pk, z, k) for z, k in zip(zs, ks)], f"mul[{count}]")
        assert_ct_equal(pk, key, key.negate(ct), [pz.negate(pk, z) for z in zs], f"negate[{count}]")


def test_device_pointer_forms_match_host_forms(gpu_key):
    """hg_dev_* on device buffers (one caller stream) give the host forms'
    bytes: encrypt_zero, randomize, add_plain, sub_plain, plain_sub, sub
    (including out aliasing a), negate."""
    import ctypes

    torch = pytest.importorskip("torch")
    key, pk, sk = gpu_key(2048, 0)
    lib, h = key.lib, key.ctx.handle
    n = 37
    prg = Prg(91)
    ms = rand_i64(prg, n, -(2 ** 40), 2 ** 40)
    ps = rand_i64(prg, n, -(2 ** 40), 2 ** 40)
    rs = pz.r_stream(92, n, pk.key_size // 2)
    r = r_limbs(pk, rs, key)
    a = key.encrypt(np.array(ms, dtype=np.int64), r)
    b = key.encrypt(np.array(ps, dtype=np.int64), r[::-1].copy())
    dev = torch.device("cuda", 0)
    st = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(st.cuda_stream)
    T = lambda x: torch.from_numpy(np.ascontiguousarray(x).view(np.int32)).to(dev)  # noqa: E731
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    H = lambda t: t.cpu().numpy().view(np.uint32)  # noqa: E731
    da, db, dr, dp = T(a), T(b), T(r), torch.from_numpy(np.array(ps, dtype=np.int64)).to(dev)
    out = torch.empty_like(da)
    with torch.cuda.stream(st):
        capi.check(lib.hg_dev_encrypt_zero(h, key.id, P(dr), P(out), n, sp))
        torch.cuda.synchronize()
        assert np.array_equal(H(out), key.encrypt_zero(r))
        rr = da.clone()
        capi.check(lib.hg_dev_randomize(h, key.id, P(rr), P(dr), n, sp))
        torch.cuda.synchronize()
        assert np.array_equal(H(rr), key.randomize(a, r))
        for fn, want in ((lib.hg_dev_add_plain, key.add_plain(a, ps)), (lib.hg_dev_sub_plain, key.sub_plain(a, ps))):
            capi.check(fn(h, key.id, P(da), P(dp), P(out), n, sp))
            torch.cuda.synchronize()
            assert np.array_equal(H(out), want)
        capi.check(lib.hg_dev_plain_sub(h, key.id, P(dp), P(da), P(out), n, sp))
        torch.cuda.synchronize()
        assert np.array_equal(H(out), key.plain_sub(ps, a))
        capi.check(lib.hg_dev_sub(h, key.id, P(da), P(db), P(out), n, sp))
        torch.cuda.synchronize()
        assert np.array_equal(H(out), key.sub(a, b))
        ac = da.clone()
        capi.check(lib.hg_dev_sub(h, key.id, P(ac), P(db), P(ac), n, sp))
        torch.cuda.synchronize()
        assert np.array_equal(H(ac), key.sub(a, b))
        capi.check(lib.hg_dev_negate(h, key.id, P(da), P(out), n, sp))
        torch.cuda.synchronize()
        assert np.array_equal(H(out), key.negate(a))
    capi.check(lib.hg_dev_check(h))
    d, _ = key.decrypt(H(ac))
    assert d.tolist() == [x - y for x, y in zip(ms, ps)]


def test_injected_allocation_failure_keeps_the_context_usable():
    """Failure injection on the host: with a device-bytes cap set, a call whose
    staging buffers would pass it fails with HG_ERR_NOMEM before any
    cudaMalloc; after the cap is lifted the same call succeeds on the same
    (fresh) context and key."""
    import ctypes

    pk, sk = oracle_key_small()
    ctx = hg.Context(0)
    try:
        key = ctx.load_key(1024, pk.n, pk.h_s, sk.p, sk.q, table_window=6)
        lib = key.lib
        held = ctypes.c_size_t()
        capi.check(lib.hg_probe_set_alloc_limit(0, ctypes.byref(held)))
        n = 4096
        m = np.arange(n, dtype=np.int64) - n // 2
        r = np.zeros((n, key.r_limbs), np.uint32)
        r[:, 0] = 1  # r = 1
        try:
            capi.check(lib.hg_probe_set_alloc_limit(held.value + 4096, None))
            with pytest.raises(hg.HgError) as ei:
                key.encrypt(m, r)
            assert ei.value.code == capi.HG_ERR_NOMEM
            assert "limit" in str(ei.value)
        finally:
            capi.check(lib.hg_probe_set_alloc_limit(0, None))
        ct = key.encrypt(m, r)
        d, ovf = key.decrypt(ct)
        assert ovf.sum() == 0 and np.array_equal(d, m)
        assert hg.limbs_to_ints(key.from_mont(ct[:2])) == [pz.encrypt(pk, int(v), 1) for v in m[:2]]
    finally:
        ctx.close()


def oracle_key_small():
    from tests.conftest import oracle_key

    return oracle_key(1024, 1)


def test_host_api_is_thread_safe(gpu_key):
    """Vectorized calls arrive from many threads at once (numpy/encryptor.cc
    parallel_for chunks); each host call takes one of the context's lanes."""
    import threading

    key, pk, sk = gpu_key(1024, 1)
    errors = []

    def worker(t):
        try:
            rng = np.random.default_rng(100 + t)
            for it in range(6):
                n = int(rng.integers(1, 3000))
                m = rng.integers(-(2 ** 50), 2 ** 50, size=n)
                r = rng.integers(0, 2 ** 32, size=(n, key.r_limbs), dtype=np.uint64).astype(np.uint32)
                ct = key.encrypt(m, r)
                k = rng.integers(-1000, 1000, size=n)
                d, ovf = key.decrypt(key.mul(key.add(ct, ct), k))
                if not (ovf.sum() == 0 and np.array_equal(d, 2 * m * k)):
                    errors.append((t, it))
        except Exception as e:  # collected for the main thread
            errors.append(repr(e))

    ths = [threading.Thread(target=worker, args=(t,)) for t in range(8)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    assert not errors, errors


def test_chunked_host_calls_match_single_lane_calls(gpu_key):
    """Host-pointer calls of >= 2^17 elements run as chunks alternating over two
    lanes; every element equals what an unchunked call gives, and an error in
    a chunk on either lane (range, non-invertible) is raised as before."""
    key, pk, sk = gpu_key(1024, 1)
    n = 3 * (1 << 16) + 123  # three chunks: lanes A, B, A
    per = -(-n // 3)
    rng = np.random.default_rng(31)
    m = rng.integers(-(2 ** 40), 2 ** 40, size=n, dtype=np.int64)
    r = rng.integers(0, 2 ** 32, size=(n, key.r_limbs), dtype=np.uint64).astype(np.uint32)
    k = rng.integers(-(2 ** 20), 2 ** 20, size=n, dtype=np.int64)
    ct = key.encrypt(m, r)
    d, ovf = key.decrypt(ct)
    assert ovf.sum() == 0 and np.array_equal(d, m)
    ct2 = key.encrypt(m[::-1].copy(), r)
    s = key.add(ct, ct2)
    ml = key.mul(ct, k)
    ez = key.encrypt_zero(r)
    rz = key.randomize(ct, r[::-1].copy())
    ap = key.add_plain(ct, k)
    for lo, hi in ((0, 5), (per - 4, per + 4), (2 * per - 3, 2 * per + 3), (n - 5, n)):
        sl = slice(lo, hi)
        assert np.array_equal(ct[sl], key.encrypt(m[sl], r[sl]))
        assert np.array_equal(s[sl], key.add(ct[sl], ct2[sl]))
        assert np.array_equal(ml[sl], key.mul(ct[sl], k[sl]))
        assert np.array_equal(ez[sl], key.encrypt_zero(r[sl]))
        assert np.array_equal(rz[sl], key.randomize(ct[sl], r[::-1][sl].copy()))
        assert np.array_equal(ap[sl], key.add_plain(ct[sl], k[sl]))
    d, _ = key.decrypt(ml)
    assert np.array_equal(d, m * k)
    bad = ct.copy()
    bad[per + 7] = 0xFFFFFFFF  # >= n^2, in the chunk on the second lane
    with pytest.raises(hg.HgError) as ei:
        key.decrypt(bad)
    assert ei.value.code == capi.HG_ERR_CT_RANGE
    with pytest.raises(hg.HgError) as ei:
        key.mul(bad, k)
    assert ei.value.code == capi.HG_ERR_CT_RANGE
    noinv = ct.copy()
    noinv[per + 9] = key.to_mont(hg.ints_to_limbs([sk.p], key.ct_limbs))[0]
    kneg = np.full(n, -3, dtype=np.int64)
    with pytest.raises(hg.HgError) as ei:
        key.mul(noinv, kneg)
    assert ei.value.code == capi.HG_ERR_NOT_INVERTIBLE
    d, _ = key.decrypt(key.mul(ct, kneg))
    assert np.array_equal(d, -3 * m)


def test_chunked_host_calls_from_threads(gpu_key):
    """Chunked calls from several threads: each takes a second lane only when
    one is free, so none waits on another."""
    import threading

    key, pk, sk = gpu_key(1024, 1)
    errors = []

    def worker(t):
        try:
            rng = np.random.default_rng(200 + t)
            n = (1 << 17) + t
            m = rng.integers(-(2 ** 50), 2 ** 50, size=n)
            r = rng.integers(0, 2 ** 32, size=(n, key.r_limbs), dtype=np.uint64).astype(np.uint32)
            d, ovf = key.decrypt(key.add(key.encrypt(m, r), key.encrypt(m, r)))
            if not (ovf.sum() == 0 and np.array_equal(d, 2 * m)):
                errors.append(t)
        except Exception as e:  # collected for the main thread
            errors.append(repr(e))

    ths = [threading.Thread(target=worker, args=(t,)) for t in range(5)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    assert not errors, errors


def test_add_on_page_locked_host_buffers(gpu_key):
    """hg_add with all three buffers page-locked reads and writes them in
    place from the kernel; results equal the copy path's (pageable buffers),
    also with out aliasing a."""
    import ctypes

    torch = pytest.importorskip("torch")
    key, pk, sk = gpu_key(2048, 0)
    n = 3000
    rng = np.random.default_rng(41)
    m = rng.integers(-(2 ** 40), 2 ** 40, size=n, dtype=np.int64)
    r = rng.integers(0, 2 ** 32, size=(n, key.r_limbs), dtype=np.uint64).astype(np.uint32)
    a = key.encrypt(m, r)
    b = key.encrypt(m[::-1].copy(), r)
    want = key.add(a, b)  # pageable numpy buffers: the copy path
    pa = torch.from_numpy(a.view(np.int32)).pin_memory()
    pb = torch.from_numpy(b.view(np.int32)).pin_memory()
    po = torch.empty_like(pa).pin_memory()
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    capi.check(key.lib.hg_add(key.ctx.handle, key.id, P(pa), P(pb), P(po), n))
    assert np.array_equal(po.numpy().view(np.uint32), want)
    capi.check(key.lib.hg_add(key.ctx.handle, key.id, P(pa), P(pb), P(pa), n))
    assert np.array_equal(pa.numpy().view(np.uint32), want)
    bad = pb.clone().pin_memory()
    bad[7] = -1  # >= n^2
    with pytest.raises(hg.HgError) as ei:
        capi.check(key.lib.hg_add(key.ctx.handle, key.id, P(po), P(bad), P(po), n))
    assert ei.value.code == capi.HG_ERR_CT_RANGE

"""heu.numpy-style layer on the GPU (heu_gb300/hnp.py), checked like the
reference's pylib numpy tests (heu/pylib/numpy_test.py): element-wise ops
with broadcasting, sum / select_sum / batch_select_sum, feature-wise bucket
sums with subgroup maps, matmul both ways — ciphertexts byte-equal to the
oracle under the same r stream, decryptions equal to integer arithmetic."""

import numpy as np
import pytest

import heu_gb300 as hg
from heu_gb300 import hnp
from oracle import paillier_z as pz
from tests.conftest import oracle_key

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def kit(gpu_ctx):
    k = hnp.setup(1024, seed=1, context=gpu_ctx, table_window=8)
    pk, sk = oracle_key(1024, 1)
    assert k.n == pk.n
    return k


def _stream(seed, bits=512, r_limbs=16):
    state = {"i": 0}
    rs = pz.r_stream(seed, 4096, bits)

    def source(count):
        out = hg.ints_to_limbs(rs[state["i"]: state["i"] + count], r_limbs)
        state["i"] += count
        return out

    return source, rs


def test_encrypt_decrypt_and_oracle_bytes(kit):
    pk, sk = oracle_key(1024, 1)
    src, rs = _stream(5)
    enc = kit.encryptor(src)
    vals = [[1, -2, 3], [2 ** 40, -(2 ** 62), 0]]
    ct = enc.encrypt(kit.array(vals))
    assert ct.shape == (2, 3)
    flat = [v for row in vals for v in row]
    want = [pz.to_mont(pk, pz.encrypt(pk, m, r)) for m, r in zip(flat, rs[:6])]
    assert hg.limbs_to_ints(ct.limbs) == want
    dec = kit.decryptor()
    assert dec.decrypt(ct).to_numpy().tolist() == vals
    big = enc.encrypt(kit.array([pk.n_half, -(pk.n_half - 1), 2 ** 100]))
    assert dec.decrypt(big).to_numpy().tolist() == [pk.n_half, -(pk.n_half - 1), 2 ** 100]
    with pytest.raises(ValueError, match="out of range"):
        enc.encrypt(kit.array([pk.n_half + 1]))
    assert dec.decrypt_in_range(ct, 63).to_numpy().tolist() == vals
    with pytest.raises(ValueError, match="range check failed"):
        dec.decrypt_in_range(ct, 40)


def test_elementwise_with_broadcasting(kit):
    enc, dec, ev = kit.encryptor(), kit.decryptor(), kit.evaluator()
    a = np.array([[1, 2, 3], [4, 5, 6]])
    b = np.array([10, -20, 30])
    ca, cb = enc.encrypt(kit.array(a)), enc.encrypt(kit.array(b))
    pb = kit.array(b)
    D = lambda c: dec.decrypt(c).to_numpy()  # noqa: E731
    assert np.array_equal(D(ev.add(ca, cb)), a + b)
    assert np.array_equal(D(ev.add(ca, pb)), a + b)
    assert np.array_equal(D(ev.add(pb, ca)), a + b)
    assert np.array_equal(D(ev.sub(ca, cb)), a - b)
    assert np.array_equal(D(ev.sub(ca, pb)), a - b)
    assert np.array_equal(D(ev.sub(pb, ca)), b - a)
    assert np.array_equal(D(ev.mul(ca, pb)), a * b)
    assert np.array_equal(D(ev.mul(pb, ca)), a * b)
    assert np.array_equal(D(ev.negate(ca)), -a)
    assert np.array_equal(ev.add(kit.array(a), pb).to_numpy(), a + b)
    assert np.array_equal(D(ev.add(ca, kit.array([[2 ** 100], [1]]))).astype(object),
                          (a.astype(object) + np.array([[2 ** 100], [1]], dtype=object)))
    with pytest.raises(ValueError, match="broadcast"):
        ev.add(ca, enc.encrypt(kit.array([1, 2])))
    r = ev.randomize(ca)
    assert np.array_equal(D(r), a) and not np.array_equal(r.limbs, ca.limbs)


def test_sums(kit):
    enc, dec, ev = kit.encryptor(), kit.decryptor(), kit.evaluator()
    x = np.arange(900).reshape(30, 30)
    cx = enc.encrypt(kit.array(x))
    D = lambda c: dec.decrypt(c).to_numpy()  # noqa: E731
    assert int(D(ev.sum(cx))) == 404550  # numpy_test.cc:111-120
    assert int(D(ev.select_sum(cx, (slice(2, 9), [1, 5, 29])))) == int(x[2:9][:, [1, 5, 29]].sum())
    assert int(D(ev.select_sum(cx, [3, 3, 7]))) == int(x[[3, 3, 7]].sum())
    assert int(D(ev.select_sum(cx, []))) == 0
    items = [[0, 1], slice(5, 20), [], [29]]
    got = D(ev.batch_select_sum(cx, items))
    assert got.tolist() == [int(x[it].sum()) for it in items]
    assert ev.select_sum(kit.array(x), [1, 2]) == int(x[[1, 2]].sum())


def test_feature_wise_bucket_sums(kit):
    enc, dec, ev = kit.encryptor(), kit.decryptor(), kit.evaluator()
    rng = np.random.default_rng(4)
    rows, cols, feats, buckets = 50, 2, 3, 5
    x = rng.integers(-1000, 1000, size=(rows, cols))
    om = rng.integers(0, buckets, size=(rows, feats))
    sub = (rng.random(rows) < 0.6).astype(np.int64)
    cx = enc.encrypt(kit.array(x))
    for cumsum in (False, True):
        out = dec.decrypt(ev.feature_wise_bucket_sum(cx, sub, om, buckets, cumsum)).to_numpy()
        want = np.zeros((feats * buckets, cols), dtype=np.int64)
        for i in np.nonzero(sub)[0]:
            for f in range(feats):
                want[f * buckets + om[i, f]] += x[i]
        if cumsum:
            want = want.reshape(feats, buckets, cols).cumsum(axis=1).reshape(-1, cols)
        assert np.array_equal(out, want)
    outs = ev.batch_feature_wise_bucket_sum(cx, [sub, 1 - sub, np.zeros(rows)], om, buckets)
    assert len(outs) == 3
    assert np.array_equal(dec.decrypt(outs[2]).to_numpy(), np.zeros((feats * buckets, cols)))


def test_matmul_both_ways(kit):
    enc, dec, ev = kit.encryptor(), kit.decryptor(), kit.evaluator()
    rng = np.random.default_rng(8)
    for m, k, n in [(3, 4, 2), (1, 5, 3), (4, 1, 1)]:  # matmul_test.cc-sized shapes
        x = rng.integers(-100, 100, size=(m, k))
        y = rng.integers(-(2 ** 15), 2 ** 15, size=(k, n))
        cx, cy = enc.encrypt(kit.array(x)), enc.encrypt(kit.array(y))
        assert np.array_equal(dec.decrypt(ev.matmul(cx, kit.array(y))).to_numpy(), x @ y)
        assert np.array_equal(dec.decrypt(ev.matmul(kit.array(x), cy)).to_numpy(), x @ y)
    v = rng.integers(-9, 9, size=4)
    cm = enc.encrypt(kit.array(rng.integers(-9, 9, size=(3, 4))))
    assert ev.matmul(cm, kit.array(v)).shape == (3,)


def test_batch_encoder_packed_ciphertexts(kit):
    """Two int64 per ciphertext (phe/encoding/batch_encoder.h): encrypt packed,
    add and sum slot-wise, scale by a small positive scalar."""
    enc, dec, ev = kit.encryptor(), kit.decryptor(), kit.evaluator()
    be = kit.batch_encoder()
    rng = np.random.default_rng(12)
    a1, b1 = rng.integers(-(2 ** 40), 2 ** 40, size=(2, 300))
    a2, b2 = rng.integers(-(2 ** 40), 2 ** 40, size=(2, 300))
    c1 = enc.encrypt_batch(a1, b1, be)
    c2 = enc.encrypt_batch(a2, b2, be)
    f, s = dec.decrypt_batch(c1, be)
    assert np.array_equal(f, a1) and np.array_equal(s, b1)
    f, s = dec.decrypt_batch(ev.add(c1, c2), be)
    assert np.array_equal(f, a1 + a2) and np.array_equal(s, b1 + b2)
    f, s = dec.decrypt_batch(ev.sum(c1), be)
    assert int(f) == int(a1.sum()) and int(s) == int(b1.sum())
    f, s = dec.decrypt_batch(ev.mul(c1, kit.array(np.full(300, 3))), be)
    assert np.array_equal(f, a1 * 3) and np.array_equal(s, b1 * 3)


@pytest.mark.parametrize("bits,seed", [(1024, 5), (2048, 0)])
def test_ou_schema_through_the_numpy_layer(gpu_ctx, bits, seed):
    """hnp.setup(schema="ou"): ciphertexts byte-equal to the OU oracle under the
    same r, and the element-wise / reduction surface equal to integer math."""
    from oracle import ou

    kit = hnp.setup(bits, seed=seed, context=gpu_ctx, table_window=8, schema="ou")
    pk = ou.PublicKey(kit.public_key["n"], kit.public_key["G"], kit.public_key["H"], kit.max_plaintext)
    sk = ou.SecretKey(*(kit.secret_key[k] for k in ("p", "q", "t", "gp_inv")))
    rng = np.random.default_rng(seed)
    a = rng.integers(-10 ** 6, 10 ** 6, size=(3, 4))
    b = rng.integers(-10 ** 6, 10 ** 6, size=(4,))
    rs = [int(v) | (1 << (kit.random_bits - 1)) for v in rng.integers(1, 2 ** 62, size=12)]
    enc = kit.encryptor(lambda count: hg.ints_to_limbs(rs[:count], kit.key.r_limbs))
    dec, ev = kit.decryptor(), kit.evaluator()
    x = enc.encrypt(kit.array(a))
    want = [ou.to_mont(pk, ou.encrypt(pk, int(m), r)) for m, r in zip(a.reshape(-1), rs)]
    assert hg.limbs_to_ints(x.limbs) == want
    assert [ou.decrypt(pk, sk, ou.from_mont(pk, c)) for c in want] == a.reshape(-1).tolist()
    enc = kit.encryptor()
    y = enc.encrypt(kit.array(b))
    assert np.array_equal(dec.decrypt(ev.add(x, y)).to_numpy(), a + b)
    assert np.array_equal(dec.decrypt(ev.sub(x, kit.array(b))).to_numpy(), a - b)
    assert np.array_equal(dec.decrypt(ev.mul(x, kit.array([3, -2, 0, 1]))).to_numpy(), a * [3, -2, 0, 1])
    assert np.array_equal(dec.decrypt(ev.negate(ev.randomize(x))).to_numpy(), -a)
    assert dec.decrypt(ev.sum(x)).to_numpy() == a.sum()
    assert np.array_equal(dec.decrypt(ev.matmul(x, kit.array(np.eye(4, 2, dtype=np.int64)))).to_numpy(),
                          a @ np.eye(4, 2, dtype=np.int64))
    big = kit.max_plaintext
    assert dec.decrypt(enc.encrypt(kit.array([big, -big]))).to_numpy().tolist() == [big, -big]
    with pytest.raises(ValueError, match="out of range"):
        enc.encrypt(kit.array([big + 1]))


def test_float_and_integer_encoders_through_the_engine(kit):
    """hnp.array(ndarray, FloatEncoder) -> Encrypt -> Add / Mul by an
    integer -> Decrypt -> to_numpy(FloatEncoder), as heu.numpy's float
    workflow (pylib numpy_test.py uses FloatEncoder the same way)."""
    fe = kit.float_encoder()
    x = np.array([[1.25, -2.5], [0.000001, 3.75]])
    y = np.array([[0.5, 0.5], [-1.0, 2.0]])
    enc, dec, ev = kit.encryptor(), kit.decryptor(), kit.evaluator()
    cx = enc.encrypt(kit.array(x, fe))
    s = ev.add(cx, kit.array(y, fe))
    got = dec.decrypt(ev.mul(s, kit.array([3, -2]))).to_numpy(fe)
    assert np.allclose(got, (x + y) * [3, -2])
    ie = kit.integer_encoder(10)
    ci = enc.encrypt(kit.array([7, -8], ie))
    assert dec.decrypt(ci).to_numpy(ie).tolist() == [7, -8]


def test_encrypt_with_audit_matches_oracle(kit):
    """EncryptWithAudit: "p:<m>,rn:<h_s^r>,c:<c>" with the Montgomery-form
    values the oracle gives for the same r (paillier_zahlen/encryptor.cc:50-54)."""
    pk, sk = oracle_key(1024, 1)
    src, rs = _stream(17)
    ct, audit = kit.encryptor(src).encrypt_with_audit(kit.array([[7, -9]]))
    assert ct.shape == (1, 2) and audit.shape == (1, 2)
    for j, m in enumerate((7, -9)):
        rn = pz.to_mont(pk, pz.encrypt_zero(pk, rs[j]))
        c = pz.to_mont(pk, pz.encrypt(pk, m, rs[j]))
        sign = "-" if m < 0 else ""
        assert audit[0, j] == f"p:{sign}{abs(m):X},rn:{rn:X},c:{c:X}"

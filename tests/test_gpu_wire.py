"""HEU's wire format on the GPU (hg_serialize / hg_deserialize and their
device forms, heu_gb300/csrc/wire_kernels.cu): bytes equal to the oracle
(oracle/wire.py, which restates numpy/matrix.h:221-310 and
phe/base/serializable_types.cc:49-122), round trips through the heu.numpy
layer as the reference's pickling tests do (heu/pylib/numpy_test.py:150-197),
and malformed input rejected."""

import ctypes

import numpy as np
import pytest

import heu_gb300 as hg
from heu_gb300 import capi, hnp
from oracle import wire

pytestmark = pytest.mark.gpu


def _colmajor_ints(limbs, shape):
    rows, cols, _ = wire.shape_to_matrix(shape)
    vals = hg.limbs_to_ints(limbs)
    return [vals[(k % rows) * cols + k // rows] for k in range(rows * cols)]


def _rand_ct(key, n, seed):
    rng = np.random.default_rng(seed)
    m = rng.integers(-(2 ** 40), 2 ** 40, size=n, dtype=np.int64)
    r = rng.integers(0, 2 ** 32, size=(n, key.r_limbs), dtype=np.uint64).astype(np.uint32)
    return key.encrypt(m, r), m


@pytest.mark.parametrize("bits", [1024, 2048, 3072])
@pytest.mark.parametrize("shape", [(), (1,), (7,), (3, 4), (2, 17), (0,), (40, 1)])
def test_serialize_equals_oracle_and_loads_back(gpu_key, bits, shape):
    key, pk, sk = gpu_key(bits, 0 if bits == 2048 else 1)
    n = int(np.prod(shape, dtype=np.int64))
    ct, _ = _rand_ct(key, n, 3 + n)
    buf = key.serialize(ct, shape)
    rows, cols, ndim = wire.shape_to_matrix(shape)
    assert buf == wire.serialize_matrix(_colmajor_ints(ct, shape), rows, cols, ndim, wire.SCHEMA_ZPAILLIER)
    back, shp = key.deserialize(buf)
    assert shp == tuple(shape) and np.array_equal(back, ct)


def test_short_magnitudes_and_zero(gpu_key):
    """Values with leading zero limbs and bytes (1, 255, 2^32, 0): the item
    lengths vary, so the scan places every later item."""
    key, pk, sk = gpu_key(2048, 0)
    vals = [0, 1, 255, 256, 2 ** 32, 2 ** 40 + 7, pk.n ** 2 - 1, 12345678901234567890]
    vals = vals * 300  # several scan blocks
    limbs = hg.ints_to_limbs(vals, key.ct_limbs)
    buf = key.serialize(limbs, (len(vals),))
    assert buf == wire.serialize_matrix(vals, len(vals), 1, 1, wire.SCHEMA_ZPAILLIER)
    back, _ = key.deserialize(buf)
    assert hg.limbs_to_ints(back) == vals
    # the oracle's bytes load too: item k of a 3 x 3 matrix is element (k % 3, k // 3)
    back, shp = key.deserialize(wire.serialize_matrix(vals[:9], 3, 3, 2, wire.SCHEMA_ZPAILLIER))
    got = hg.limbs_to_ints(back)
    assert shp == (3, 3) and all(got[r * 3 + c] == vals[c * 3 + r] for r in range(3) for c in range(3))


def test_numpy_layer_round_trip_decrypts(gpu_ctx):
    """numpy_test.py:150-197: serialize -> load -> decrypt gives the values."""
    kit = hnp.setup(1024, seed=4, context=gpu_ctx, table_window=8)
    enc, dec, ev = kit.encryptor(), kit.decryptor(), kit.evaluator()
    a = np.arange(-6, 6, dtype=np.int64).reshape(3, 4)
    x = enc.encrypt(kit.array(a))
    y = hnp.CiphertextArray.load_from(x.serialize(), kit)
    assert y.shape == (3, 4)
    assert np.array_equal(dec.decrypt(y).to_numpy(), a)
    s = hnp.CiphertextArray.load_from(ev.sum(x).serialize(), kit)
    assert s.shape == () and int(dec.decrypt(s).to_numpy()) == int(a.sum())


def test_ou_items_carry_the_ou_schema(gpu_ctx):
    kit = hnp.setup(2048, seed=0, context=gpu_ctx, table_window=8, schema="ou")
    x = kit.encryptor().encrypt(kit.array([1, -2, 3]))
    buf = x.serialize()
    rows, cols, ndim, vals, schemas = wire.parse_matrix(buf)
    assert (rows, cols, ndim) == (3, 1, 1) and schemas == [wire.SCHEMA_OU] * 3
    assert vals == hg.limbs_to_ints(x.limbs)
    y = hnp.CiphertextArray.load_from(buf, kit)
    assert kit.decryptor().decrypt(y).to_numpy().tolist() == [1, -2, 3]


def test_malformed_and_mismatched_input_is_rejected(gpu_key, gpu_ctx):
    key, pk, sk = gpu_key(1024, 1)
    ct, _ = _rand_ct(key, 6, 9)
    buf = key.serialize(ct, (2, 3))
    cases = [buf[:-1], buf[:5], b"\x93" + buf[1:], b"", buf[:1] + b"\x03" + buf[2:]]
    # an item whose schema byte is OU's under a ZPaillier key
    cases.append(wire.serialize_matrix(hg.limbs_to_ints(ct), 6, 1, 1, wire.SCHEMA_OU))
    # an item with more magnitude bytes than the key's limbs hold
    cases.append(wire.serialize_matrix([1 << (32 * key.ct_limbs)], 1, 1, 1, wire.SCHEMA_ZPAILLIER))
    # an item whose c_ is a str instead of a bin
    it = wire.item_bytes(5, 4)
    bad_item = b"\x91\xa1\x05" + it[-8:]
    cases.append(b"\x94\x01\x01\x01\x91" + wire._str_header(len(bad_item)) + bad_item)
    for bad in cases:
        with pytest.raises(hg.HgError) as ei:
            key.deserialize(bad)
        assert ei.value.code == capi.HG_ERR_INVALID
    # too small an output buffer: nothing written, the size needed reported
    lib, h = key.lib, key.ctx.handle
    out = np.zeros(10, np.uint8)
    ln = ctypes.c_size_t()
    P = lambda a: ctypes.c_void_p(a.ctypes.data)  # noqa: E731
    rc = lib.hg_serialize(h, key.id, P(ct), 2, 3, 2, 1, P(out), out.size, ctypes.byref(ln))
    assert rc == capi.HG_ERR_INVALID and ln.value == len(buf) and not out.any()
    # the context still works
    back, shp = key.deserialize(buf)
    assert np.array_equal(back, ct)


def test_device_forms_match_host_forms(gpu_key):
    torch = pytest.importorskip("torch")
    key, pk, sk = gpu_key(2048, 0)
    ct, _ = _rand_ct(key, 1000, 12)
    buf = key.serialize(ct, (40, 25))
    lib, h = key.lib, key.ctx.handle
    dev = torch.device("cuda", 0)
    st = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(st.cuda_stream)
    dct = torch.from_numpy(ct.view(np.int32)).to(dev)
    bound = ctypes.c_size_t()
    capi.check(lib.hg_serialize_bound(h, key.id, 1000, ctypes.byref(bound)))
    dout = torch.empty(bound.value, dtype=torch.uint8, device=dev)
    ln = ctypes.c_size_t()
    capi.check(lib.hg_dev_serialize(h, key.id, ctypes.c_void_p(dct.data_ptr()), 40, 25, 2, 1,
                                    ctypes.c_void_p(dout.data_ptr()), bound.value, ctypes.byref(ln), sp))
    assert ln.value == len(buf) and dout[:ln.value].cpu().numpy().tobytes() == buf
    # ciphertexts at an address that is 4-byte but not 16-byte aligned
    shifted = torch.zeros(dct.numel() + 1, dtype=torch.int32, device=dev)
    shifted[1:].copy_(dct.reshape(-1))
    dout.zero_()
    capi.check(lib.hg_dev_serialize(h, key.id, ctypes.c_void_p(shifted.data_ptr() + 4), 40, 25, 2, 1,
                                    ctypes.c_void_p(dout.data_ptr()), bound.value, ctypes.byref(ln), sp))
    assert dout[:ln.value].cpu().numpy().tobytes() == buf
    back = torch.empty_like(dct)
    b = np.frombuffer(buf, np.uint8)
    rows, cols, nd = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_int()
    capi.check(lib.hg_dev_deserialize(h, key.id, ctypes.c_void_p(b.ctypes.data), b.size, 1,
                                      ctypes.c_void_p(back.data_ptr()), 1000, ctypes.byref(rows), ctypes.byref(cols),
                                      ctypes.byref(nd), sp))
    capi.check(lib.hg_dev_check(h))
    assert (rows.value, cols.value, nd.value) == (40, 25, 2)
    assert np.array_equal(back.cpu().numpy().view(np.uint32), ct)


def test_full_size_round_trip(gpu_key):
    """2^20 ciphertexts at 2048 bits: serialize -> deserialize is the
    identity, the size is the sum of the item sizes, and items parse."""
    key, pk, sk = gpu_key(2048, 0)
    n = 1 << 20
    rng = np.random.default_rng(21)
    ct = rng.integers(0, 2 ** 32, size=(n, key.ct_limbs), dtype=np.uint64).astype(np.uint32)
    ct[::7, -1] = 0  # some shorter magnitudes
    ct[::11, -3:] = 0
    buf = key.serialize(ct, (n,))
    back, shp = key.deserialize(buf)
    assert shp == (n,) and np.array_equal(back, ct)
    # exact size: prefix + per item str header + [bin] + 8
    nz = ct != 0
    top = key.ct_limbs - 1 - np.argmax(nz[:, ::-1], axis=1)
    topv = ct[np.arange(n), top].astype(np.int64)
    b = top.astype(np.int64) * 4 + 1 + (topv >= 1 << 8) + (topv >= 1 << 16) + (topv >= 1 << 24)
    inner = 1 + np.where(b < 256, 2, 3) + b + 8
    items = np.where(inner < 256, 2, 3) + inner
    prefix = b"\x94" + wire._uint(n) + wire._uint(1) + wire._uint(1) + wire._array_header(n)
    assert len(buf) == len(prefix) + int(items.sum()) and buf.startswith(prefix)
    assert wire.parse_item(buf[-int(inner[-1]):]) == (hg.limbs_to_ints(ct[-1:])[0], 4)


def test_pickling_and_public_key_kits(gpu_ctx):
    """heu/pylib/phe_test.py:256-270 flow: a client pickles ciphertexts, a
    server set up from the client's public key evaluates on them without the
    secret key, the client unpickles the result and decrypts."""
    import pickle

    client = hnp.setup(1024, seed=6, context=gpu_ctx, table_window=8)
    server = hnp.setup(dict(client.public_key), context=gpu_ctx, table_window=8)
    assert server.secret_key is None and server.n == client.n
    with pytest.raises(ValueError):
        server.decryptor()
    a = np.array([[1, -2], [3, 4]])
    x = client.encryptor().encrypt(client.array(a))
    y = pickle.loads(pickle.dumps(x))
    assert y.kit is client and np.array_equal(y.limbs, x.limbs)
    on_server = hnp.CiphertextArray.load_from(x.serialize(), server)
    ev = server.evaluator()
    z = ev.mul(ev.add(on_server, server.encryptor().encrypt(server.array([10, 20]))), server.array([2, 3]))
    back = pickle.loads(pickle.dumps(z))
    assert back.kit is client
    assert np.array_equal(client.decryptor().decrypt(back).to_numpy(), (a + [10, 20]) * [2, 3])
    ou_client = hnp.setup(1024, seed=2, context=gpu_ctx, table_window=8, schema="ou")
    ou_server = hnp.setup(dict(ou_client.public_key), context=gpu_ctx, table_window=8)
    assert ou_server.schema == "ou" and ou_server.secret_key is None
    c = ou_server.encryptor().encrypt(ou_server.array([5, -6]))
    assert ou_client.decryptor().decrypt(pickle.loads(pickle.dumps(c))).to_numpy().tolist() == [5, -6]

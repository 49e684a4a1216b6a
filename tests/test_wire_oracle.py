"""The wire-format oracle (oracle/wire.py) against an independent msgpack
implementation: every layer the reference fixes (numpy/matrix.h:221-310,
phe/base/serializable_types.cc:49-122, util/he_object.h:27-36) decodes with
msgpack-python to the expected objects, and the bytes equal msgpack-python's
own packing of the same objects where the two libraries' rules coincide."""

import random
import struct

import pytest

from oracle import wire


def _vals(rng, n, bits):
    return [rng.getrandbits(bits) for _ in range(n)]


@pytest.mark.parametrize("rows,cols,ndim", [(1, 1, 0), (7, 1, 1), (3, 4, 2), (200, 1, 1), (17, 5, 2), (0, 1, 1)])
def test_layers_decode_with_msgpack(rows, cols, ndim):
    msgpack = pytest.importorskip("msgpack")
    rng = random.Random(rows * 31 + cols)
    vals = _vals(rng, rows * cols, 4096)
    if vals:
        vals[0] = 0  # empty magnitude
    if len(vals) > 2:
        vals[1], vals[2] = 1, 255
    buf = wire.serialize_matrix(vals, rows, cols, ndim, wire.SCHEMA_ZPAILLIER)
    top = msgpack.unpackb(buf, raw=True)
    assert top[:3] == [rows, cols, ndim] and len(top[3]) == rows * cols
    for v, item in zip(vals, top[3]):
        assert item[-8:] == struct.pack("<Q", 4)
        (mag,) = msgpack.unpackb(item[:-8], raw=True)
        assert int.from_bytes(mag, "little") == v
        assert mag == v.to_bytes((v.bit_length() + 7) // 8, "little")
    assert wire.parse_matrix(buf) == (rows, cols, ndim, vals, [4] * len(vals))


def test_bytes_equal_msgpack_python_packing():
    """Items of 256..65535 bytes (every 1024..3072-bit ciphertext) use the same
    headers in msgpack-c and in msgpack-python's raw mode; integers and arrays
    use the smallest form in both."""
    msgpack = pytest.importorskip("msgpack")
    rng = random.Random(5)
    for rows, cols, ndim, bits in ((3, 4, 2, 2048), (70000, 1, 1, 4096), (300, 2, 2, 6144)):
        vals = [v | (1 << (bits - 1)) for v in _vals(rng, rows * cols, bits)]
        items = [msgpack.packb([v.to_bytes((v.bit_length() + 7) // 8, "little")], use_bin_type=True)
                 + struct.pack("<Q", 1) for v in vals]
        want = msgpack.packb([rows, cols, ndim, items], use_bin_type=False)
        assert wire.serialize_matrix(vals, rows, cols, ndim, wire.SCHEMA_OU) == want


def test_header_forms_at_the_boundaries():
    assert wire._uint(127) == b"\x7f" and wire._uint(128) == b"\xcc\x80"
    assert wire._uint(65535) == b"\xcd\xff\xff" and wire._uint(65536) == b"\xce\x00\x01\x00\x00"
    assert wire._array_header(15) == b"\x9f" and wire._array_header(16) == b"\xdc\x00\x10"
    assert wire._array_header(65536) == b"\xdd\x00\x01\x00\x00"
    assert wire._str_header(31) == b"\xbf" and wire._str_header(32) == b"\xd9\x20"
    assert wire._str_header(256) == b"\xda\x01\x00"
    assert wire.item_bytes(0, 4) == b"\x91\xc4\x00" + struct.pack("<Q", 4)


def test_parse_rejects_malformed_buffers():
    buf = wire.serialize_matrix([5, 6], 2, 1, 1, 4)
    for bad in (buf[:-1], b"\x93" + buf[1:], buf[:4] + b"\x93" + buf[5:], b""):
        with pytest.raises(wire.WireError):
            wire.parse_matrix(bad)
    it = wire.item_bytes(7, 4)
    with pytest.raises(wire.WireError):
        wire.parse_item(b"\x92" + it[1:])
    with pytest.raises(wire.WireError):
        wire.parse_item(it[:3])


def test_shape_mapping():
    assert wire.shape_to_matrix(()) == (1, 1, 0)
    assert wire.shape_to_matrix((5,)) == (5, 1, 1)
    assert wire.shape_to_matrix((2, 3)) == (2, 3, 2)
    with pytest.raises(wire.WireError):
        wire.shape_to_matrix((1, 2, 3))

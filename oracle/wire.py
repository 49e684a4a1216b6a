"""CPU restatement of HEU's wire format for ciphertext matrices.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` as the checker, never by the
shipped engine.

Layers, each from the reference (paths relative to the HEU project root):

  matrix      heu/library/numpy/matrix.h:221-262 (Serialize), 264-310 (LoadFrom):
              msgpack array(4) [rows, cols, ndim, array(n) of items], items
              packed from std::string_view, i.e. msgpack str; element order
              is the DenseMatrix storage order, column-major (matrix.h:159-162)
  item        phe/base/serializable_types.cc:49-69 (Serialize), 113-122
              (Deserialize): the class bytes, then the SchemaType value as a
              little-endian size_t; the reader takes its low byte
  class       util/he_object.h:27-36 (msgpack::pack of the class) with
              MSGPACK_DEFINE(c_) (paillier_zahlen/ciphertext.h:38,
              ou/ciphertext.h:38): a one-element array [c_]
  schema      phe/base/schema.h:47-51: OU = 1, ZPaillier = 4

The msgpack rules are those of msgpack-c 6.1.0 (the reference's pinned
dependency, not vendored): non-negative integers in the smallest of positive
fixint / uint8 / uint16 / uint32 / uint64, str in fixstr / str8 / str16 /
str32, arrays in fixarray / array16 / array32, all lengths big-endian.

The BigInt field c_ is encoded by yacl's msgpack adaptor, which is not in
the reference tree; this restatement (and the engine) writes it as a msgpack
bin of the little-endian magnitude without leading zero bytes.  That one
field's bytes are therefore unpinned against the reference; every layer
around it follows the reference's code.
"""

import struct

SCHEMA_OU = 1
SCHEMA_ZPAILLIER = 4


class WireError(ValueError):
    pass


def _uint(v):
    if v < 0:
        raise WireError("negative integer")
    if v < 128:
        return bytes([v])
    if v < 1 << 8:
        return b"\xcc" + struct.pack(">B", v)
    if v < 1 << 16:
        return b"\xcd" + struct.pack(">H", v)
    if v < 1 << 32:
        return b"\xce" + struct.pack(">I", v)
    return b"\xcf" + struct.pack(">Q", v)


def _array_header(n):
    if n < 16:
        return bytes([0x90 | n])
    if n < 1 << 16:
        return b"\xdc" + struct.pack(">H", n)
    return b"\xdd" + struct.pack(">I", n)


def _str_header(n):
    if n < 32:
        return bytes([0xA0 | n])
    if n < 1 << 8:
        return b"\xd9" + struct.pack(">B", n)
    if n < 1 << 16:
        return b"\xda" + struct.pack(">H", n)
    return b"\xdb" + struct.pack(">I", n)


def _bin(data):
    n = len(data)
    if n < 1 << 8:
        return b"\xc4" + struct.pack(">B", n) + data
    if n < 1 << 16:
        return b"\xc5" + struct.pack(">H", n) + data
    return b"\xc6" + struct.pack(">I", n) + data


def item_bytes(c, schema):
    """One ciphertext: msgpack [c] + schema as little-endian size_t."""
    if c < 0:
        raise WireError("negative ciphertext")
    mag = c.to_bytes((c.bit_length() + 7) // 8, "little")
    return b"\x91" + _bin(mag) + struct.pack("<Q", schema)


def serialize_matrix(values, rows, cols, ndim, schema):
    """values: rows * cols ints in column-major (storage) order."""
    if len(values) != rows * cols:
        raise WireError("rows * cols != number of values")
    out = [b"\x94", _uint(rows), _uint(cols), _uint(ndim), _array_header(len(values))]
    for v in values:
        it = item_bytes(int(v), schema)
        out.append(_str_header(len(it)))
        out.append(it)
    return b"".join(out)


class _Reader:
    def __init__(self, buf):
        self.b = buf
        self.i = 0

    def take(self, n):
        if self.i + n > len(self.b):
            raise WireError("truncated")
        v = self.b[self.i:self.i + n]
        self.i += n
        return v

    def byte(self):
        return self.take(1)[0]

    def be(self, n):
        return int.from_bytes(self.take(n), "big")

    def integer(self):
        t = self.byte()
        if t < 0x80:
            return t
        if t >= 0xE0:
            return t - 256
        if 0xCC <= t <= 0xCF:
            return self.be(1 << (t - 0xCC))
        if 0xD0 <= t <= 0xD3:
            n = 1 << (t - 0xD0)
            return int.from_bytes(self.take(n), "big", signed=True)
        raise WireError("integer")

    def array(self):
        t = self.byte()
        if t & 0xF0 == 0x90:
            return t & 0x0F
        if t == 0xDC:
            return self.be(2)
        if t == 0xDD:
            return self.be(4)
        raise WireError("array")

    def raw(self):
        t = self.byte()
        if t & 0xE0 == 0xA0:
            n = t & 0x1F
        elif t in (0xD9, 0xC4):
            n = self.be(1)
        elif t in (0xDA, 0xC5):
            n = self.be(2)
        elif t in (0xDB, 0xC6):
            n = self.be(4)
        else:
            raise WireError("str/bin")
        return self.take(n)


def parse_item(it):
    """-> (c, schema low byte)."""
    if len(it) <= 8:
        raise WireError("item too short")
    r = _Reader(it[:-8])
    if r.array() != 1:
        raise WireError("class is not a one-element array")
    t = r.b[r.i]
    if t not in (0xC4, 0xC5, 0xC6):
        raise WireError("c_ is not a bin")
    mag = r.raw()
    if r.i != len(r.b):
        raise WireError("trailing bytes in item")
    return int.from_bytes(mag, "little"), it[-8]


def parse_matrix(buf):
    """-> (rows, cols, ndim, values in column-major order, schema bytes)."""
    r = _Reader(buf)
    if r.array() != 4:
        raise WireError("not a 4-element array")
    rows, cols, ndim = r.integer(), r.integer(), r.integer()
    n = r.array()
    if n != rows * cols:
        raise WireError("inner array size != rows * cols")
    vals, schemas = [], []
    for _ in range(n):
        c, s = parse_item(r.raw())
        vals.append(c)
        schemas.append(s)
    return rows, cols, ndim, vals, schemas


def shape_to_matrix(shape):
    """NumPy shape -> (rows, cols, ndim) as heu.numpy keeps it: a scalar is
    1 x 1, a vector n x 1 (numpy/shape.h:44-54 RowsAlloc / ColsAlloc)."""
    if len(shape) == 0:
        return 1, 1, 0
    if len(shape) == 1:
        return shape[0], 1, 1
    if len(shape) == 2:
        return shape[0], shape[1], 2
    raise WireError("heu.numpy arrays have at most 2 dimensions")

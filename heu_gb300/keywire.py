"""HEU's wire format for keys, on the host.

A key serializes like every HeObject (heu/library/algorithms/util/
he_object.h:27-36): the msgpack of the class, then, through phe's
SerializableVariant, the schema value as a little-endian size_t
(phe/base/serializable_types.cc:49-69; 4 = ZPaillier, 1 = OU,
phe/base/schema.h:47-51).  The classes' msgpack layouts:

  ZPaillier PublicKey  [n, h_s]                      paillier_zahlen/public_key.h:60-93
  ZPaillier SecretKey  [lambda, mu, p, q]            paillier_zahlen/secret_key.h:60-93
                       lambda = (p-1)(q-1)/2, mu = lambda^-1 mod n (key_generator.cc:53-54)
  OU PublicKey         [n, G, H, bits(max_plaintext) - 1]   ou/public_key.h:134-165
  OU SecretKey         [p, q, t, gp_inv, p^2, p/2, n]       ou/secret_key.h:37

BigInt fields are written as a msgpack bin of the little-endian magnitude
(the same choice as the ciphertext wire format: yacl's BigInt adaptor is not
in the reference tree), the size_t as the smallest msgpack unsigned int.
Keys are small, so this is plain Python.
"""

import struct

SCHEMA_OU = 1
SCHEMA_ZPAILLIER = 4


class KeyFormatError(ValueError):
    pass


# ---- msgpack pieces (msgpack-c's smallest forms) ---------------------------
def _uint(v):
    if v < 128:
        return bytes([v])
    for tag, fmt, lim in ((0xCC, ">B", 1 << 8), (0xCD, ">H", 1 << 16), (0xCE, ">I", 1 << 32)):
        if v < lim:
            return bytes([tag]) + struct.pack(fmt, v)
    return b"\xcf" + struct.pack(">Q", v)


def _bigint(v):
    if v < 0:
        raise KeyFormatError("key fields are non-negative")
    mag = v.to_bytes((v.bit_length() + 7) // 8, "little")
    n = len(mag)
    if n < 1 << 8:
        return b"\xc4" + struct.pack(">B", n) + mag
    if n < 1 << 16:
        return b"\xc5" + struct.pack(">H", n) + mag
    return b"\xc6" + struct.pack(">I", n) + mag


def _array(items):
    n = len(items)
    head = bytes([0x90 | n]) if n < 16 else b"\xdc" + struct.pack(">H", n)
    return head + b"".join(items)


class _Reader:
    def __init__(self, buf):
        self.b, self.i = buf, 0

    def take(self, n):
        if self.i + n > len(self.b):
            raise KeyFormatError("truncated key")
        v = self.b[self.i:self.i + n]
        self.i += n
        return v

    def byte(self):
        return self.take(1)[0]

    def array(self):
        t = self.byte()
        if t & 0xF0 == 0x90:
            return t & 0x0F
        if t == 0xDC:
            return int.from_bytes(self.take(2), "big")
        raise KeyFormatError("not an array")

    def bigint(self):
        t = self.byte()
        widths = {0xC4: 1, 0xC5: 2, 0xC6: 4}
        if t not in widths:
            raise KeyFormatError("BigInt field is not a bin")
        n = int.from_bytes(self.take(widths[t]), "big")
        return int.from_bytes(self.take(n), "little")

    def uint(self):
        t = self.byte()
        if t < 0x80:
            return t
        widths = {0xCC: 1, 0xCD: 2, 0xCE: 4, 0xCF: 8}
        if t not in widths:
            raise KeyFormatError("not an unsigned integer")
        return int.from_bytes(self.take(widths[t]), "big")


def _with_schema(payload, schema):
    return payload + struct.pack("<Q", schema)


def _split(buf):
    buf = bytes(buf)
    if len(buf) <= 8:
        raise KeyFormatError("key buffer too short")
    return buf[:-8], buf[-8]  # serializable_types.cc:117 reads the low byte


# ---- public keys -------------------------------------------------------------
def serialize_public_key(pk, schema):
    """pk: a kit's ``public_key`` dict; schema "zpaillier" or "ou"."""
    if schema == "ou":
        body = _array([_bigint(pk["n"]), _bigint(pk["G"]), _bigint(pk["H"]), _uint(pk["max_pt_bits"])])
        return _with_schema(body, SCHEMA_OU)
    return _with_schema(_array([_bigint(pk["n"]), _bigint(pk["h_s"])]), SCHEMA_ZPAILLIER)


def deserialize_public_key(buf):
    """-> (schema, public_key dict) as ``hnp.setup(public_key)`` takes it."""
    body, schema = _split(buf)
    r = _Reader(body)
    k = r.array()
    if schema == SCHEMA_OU:
        if k != 4:
            raise KeyFormatError("OU public key is a 4-element array")
        pk = {"n": r.bigint(), "G": r.bigint(), "H": r.bigint(), "max_pt_bits": r.uint()}
        out = "ou"
    elif schema == SCHEMA_ZPAILLIER:
        if k != 2:
            raise KeyFormatError("ZPaillier public key is a 2-element array")
        pk = {"n": r.bigint(), "h_s": r.bigint()}
        out = "zpaillier"
    else:
        raise KeyFormatError(f"schema value {schema} is neither ZPaillier (4) nor OU (1)")
    if r.i != len(body):
        raise KeyFormatError("trailing bytes in key")
    return out, pk


# ---- secret keys -------------------------------------------------------------
def serialize_secret_key(sk, n, schema):
    """sk: a kit's ``secret_key`` dict, n its modulus."""
    if schema == "ou":
        p, q = sk["p"], sk["q"]
        fields = [p, q, sk["t"], sk["gp_inv"], p * p, p >> 1, n]
        return _with_schema(_array([_bigint(v) for v in fields]), SCHEMA_OU)
    p, q = sk["p"], sk["q"]
    lam = (p - 1) * (q - 1) // 2
    mu = pow(lam, -1, n)
    return _with_schema(_array([_bigint(v) for v in (lam, mu, p, q)]), SCHEMA_ZPAILLIER)


def deserialize_secret_key(buf):
    """-> (schema, secret_key dict with the fields the engine loads)."""
    body, schema = _split(buf)
    r = _Reader(body)
    k = r.array()
    if schema == SCHEMA_OU:
        if k != 7:
            raise KeyFormatError("OU secret key is a 7-element array")
        p, q, t, gp_inv, p2, phalf, n = (r.bigint() for _ in range(7))
        if p2 != p * p or phalf != p >> 1 or n != p * p * q:
            raise KeyFormatError("OU secret key fields disagree")
        out, sk = "ou", {"p": p, "q": q, "t": t, "gp_inv": gp_inv, "n": n}
    elif schema == SCHEMA_ZPAILLIER:
        if k != 4:
            raise KeyFormatError("ZPaillier secret key is a 4-element array")
        lam, mu, p, q = (r.bigint() for _ in range(4))
        if lam != (p - 1) * (q - 1) // 2 or (lam * mu) % (p * q) != 1:
            raise KeyFormatError("ZPaillier secret key fields disagree")
        out, sk = "zpaillier", {"p": p, "q": q}
    else:
        raise KeyFormatError(f"schema value {schema} is neither ZPaillier (4) nor OU (1)")
    if r.i != len(body):
        raise KeyFormatError("trailing bytes in key")
    return out, sk

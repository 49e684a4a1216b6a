"""heu.numpy-style tensors over the engine.

Mirrors the Python surface of HEU's heu.numpy module for this schema
(heu/pylib/numpy_binding/bind_numpy.cc:381-480, extension_functions.cc:28-138):
``setup`` returns a kit with ``encryptor()``, ``decryptor()``, ``evaluator()``
and ``array()``; the evaluator offers add / sub / mul (with NumPy broadcasting
of the two shapes, numpy/evaluator.cc:160-185), matmul, sum, select_sum,
batch_select_sum, feature_wise_bucket_sum and batch_feature_wise_bucket_sum.

Two schemes: ZPaillier (the default) and OU (``setup(..., schema="ou")``,
heu/library/algorithms/ou), both on the same kernels.  Plaintexts are
integers (int64 NumPy arrays, or Python ints up to the scheme's plaintext
bound in an object array), or floats / scaled integers through
``FloatEncoder`` / ``IntegerEncoder``; ``BatchEncoder`` packs two int64
values per plaintext.  Ciphertexts are kept as a (size, S) uint32 limb array in
Montgomery form with a logical shape, exactly the bytes the C-ABI exchanges.
"""

import os
import weakref

import numpy as np

from heu_gb300 import engine, keywire

_I64_MIN, _I64_MAX = -(2 ** 63), 2 ** 63 - 1


def _hex(v):
    return ("-" if v < 0 else "") + format(abs(v), "X")


def _as_values(values):
    a = np.asarray(values, dtype=object) if not isinstance(values, np.ndarray) else values
    if a.dtype != object:
        return np.asarray(a, dtype=np.int64)
    flat = [int(v) for v in a.reshape(-1)]
    if all(_I64_MIN <= v <= _I64_MAX for v in flat):
        return np.array(flat, dtype=np.int64).reshape(a.shape)
    out = np.empty(len(flat), dtype=object)
    out[:] = flat
    return out.reshape(a.shape)



def _matmul_plain(values):
    """Plaintext operand of MatMul: int64 when every entry fits, else an
    object array of Python ints (the engine then takes the multi-limb path)."""
    v = np.asarray(values)
    if v.dtype != object:
        return np.asarray(v, dtype=np.int64)
    if all(-(2 ** 63) <= int(e) < 2 ** 63 for e in v.reshape(-1)):
        return np.array([int(e) for e in v.reshape(-1)], dtype=np.int64).reshape(v.shape)
    return v

class PlaintextArray:
    """Integer tensor (int64 or object dtype for values beyond int64)."""

    def __init__(self, values):
        self.values = _as_values(values)

    @property
    def shape(self):
        return self.values.shape

    @property
    def ndim(self):
        return self.values.ndim

    @property
    def size(self):
        return self.values.size

    def __getitem__(self, item):
        return PlaintextArray(self.values[item])

    def to_numpy(self, encoder=None):
        """The values, or the values decoded by ``encoder`` (heu.numpy
        PMatrix.to_numpy(encoder), bind_numpy.cc:75-92)."""
        return encoder.decode(self.values) if encoder is not None else self.values.copy()

    def __str__(self):
        return str(self.values)

    __repr__ = __str__


class EncodedArray(PlaintextArray):
    """hnp.array(values, encoder) for an IntegerEncoder / FloatEncoder: the
    raw values and their encoder.  Encryption encodes them on the device
    (the engine's PlainEncoder codec), so no host encode pass runs; the
    encoded integers are computed on the host only if ``values`` is read."""

    def __init__(self, raw, encoder):
        self.raw = np.asarray(raw)
        self.encoder = encoder
        self._values = None

    @property
    def values(self):
        if self._values is None:
            self._values = _as_values(self.encoder.encode(self.raw))
        return self._values

    @property
    def shape(self):
        return self.raw.shape

    @property
    def ndim(self):
        return self.raw.ndim

    @property
    def size(self):
        return self.raw.size

    def __getitem__(self, item):
        return EncodedArray(self.raw[item], self.encoder)

    def device_codec(self):
        """(codec, raw values) when the device can encode them, else None."""
        if type(self.encoder) not in (IntegerEncoder, FloatEncoder):
            return None
        if self.raw.dtype.kind == "f":
            return engine.capi.HG_CODEC_PLAIN_F64, self.raw.astype(np.float64)
        if self.raw.dtype.kind in "iu" and (self.raw.size == 0 or (int(self.raw.max()) < 2 ** 63 and
                                                                    int(self.raw.min()) >= -(2 ** 63))):
            return engine.capi.HG_CODEC_PLAIN_I64, self.raw.astype(np.int64)
        return None


class DecryptedArray(PlaintextArray):
    """Decryptor.decrypt's result: the plaintexts of a ciphertext array,
    decrypted when ``values`` is read; ``to_numpy(encoder)`` with an
    IntegerEncoder / FloatEncoder decrypts and decodes in one device pass
    (the engine's PlainEncoder codec)."""

    def __init__(self, decryptor, ct):
        self._dec = decryptor
        self._ct = ct
        self._values = None

    @property
    def values(self):
        if self._values is None:
            self._values = self._dec._decrypt_values(self._ct)
        return self._values

    @property
    def shape(self):
        return self._ct.shape

    @property
    def ndim(self):
        return self._ct.ndim

    @property
    def size(self):
        return self._ct.size

    def __getitem__(self, item):
        return DecryptedArray(self._dec, self._ct[item])

    def to_numpy(self, encoder=None):
        kit = self._dec.kit
        if (encoder is not None and type(encoder) in (IntegerEncoder, FloatEncoder) and kit.schema == "zpaillier"
                and self._values is None and self._ct.size > 0):
            codec = engine.capi.HG_CODEC_PLAIN_F64 if type(encoder) is FloatEncoder else engine.capi.HG_CODEC_PLAIN_I64
            out, ovf = kit.key.decrypt_decoded(codec, encoder.scale, self._ct.limbs)
            if not ovf.any():
                return out.reshape(self.shape)
        return super().to_numpy(encoder)


class CiphertextArray:
    """Ciphertext tensor: limbs (size, S) in Montgomery form plus a shape."""

    def __init__(self, kit, limbs, shape):
        self.kit = kit
        self.limbs = np.ascontiguousarray(limbs, dtype=np.uint32).reshape(-1, kit.key.ct_limbs)
        self.shape = tuple(shape)
        if int(np.prod(self.shape, dtype=np.int64)) != self.limbs.shape[0]:
            raise ValueError("shape does not match the number of ciphertexts")

    @property
    def ndim(self):
        return len(self.shape)

    @property
    def size(self):
        return self.limbs.shape[0]

    def __len__(self):
        return self.shape[0]

    def __getitem__(self, item):
        idx = np.arange(self.size).reshape(self.shape)[item]
        idx = np.asarray(idx)
        return CiphertextArray(self.kit, self.limbs[idx.reshape(-1)], idx.shape)

    def __setitem__(self, item, value):
        """x[item] = ciphertexts (a CiphertextArray of the same key), with
        NumPy's indexing and broadcasting (bind_numpy.cc __setitem__)."""
        if not isinstance(value, CiphertextArray):
            raise TypeError("only ciphertexts can be assigned into a CiphertextArray")
        sel = np.asarray(np.arange(self.size).reshape(self.shape)[item])
        src = np.broadcast_to(np.arange(value.size).reshape(value.shape), sel.shape)
        self.limbs[sel.reshape(-1)] = value.limbs[src.reshape(-1)]

    def transpose(self):
        """DenseMatrix::Transpose (numpy/matrix.h:203-206): 2-d arrays only."""
        if self.ndim != 2:
            raise ValueError(f"you cannot transpose a {self.ndim}d-tensor")
        idx = np.arange(self.size).reshape(self.shape).T.reshape(-1)
        return CiphertextArray(self.kit, self.limbs[idx], self.shape[::-1])

    @property
    def T(self):
        return self.transpose()

    def grid(self):
        """limbs as (*shape, S)"""
        return self.limbs.reshape(self.shape + (self.kit.key.ct_limbs,))

    def __str__(self):
        return f"CiphertextArray(shape={self.shape}, key_bits={self.kit.key.key_bits})"

    __repr__ = __str__

    def serialize(self):
        """DenseMatrix::Serialize (numpy/matrix.h:221-262, pylib ``serialize``):
        HEU's msgpack layout, packed on the GPU."""
        return self.kit.key.serialize(self.limbs, self.shape)

    def __reduce__(self):
        # pickling (pylib PickleSupport): the wire bytes plus the key's n
        return _unpickle_ciphertexts, (self.serialize(), self.kit.n)

    @staticmethod
    def load_from(bytes_buffer, kit):
        """DenseMatrix::LoadFrom (numpy/matrix.h:264-310, pylib ``load_from``).
        Unlike the reference, the items are turned back into limbs by the
        engine of ``kit``'s key, so the kit is an argument."""
        limbs, shape = kit.key.deserialize(bytes_buffer)
        return CiphertextArray(kit, limbs, shape)


class IntegerEncoder:
    """PlainEncoder (phe/encoding/plain_encoder.h:46-74) as pylib's
    IntegerEncoder: encode = value * scale (integers exactly, floats as the
    double product truncated toward zero, as a BigInt built from a double);
    decode = value / scale with C++ integer division (toward zero)."""

    def __init__(self, scale=1):
        self.scale = int(scale)
        if self.scale <= 0:
            raise ValueError("scale must be positive")

    def encode(self, values):
        a = np.asarray(values)
        s = self.scale
        if a.dtype.kind == "f":
            r = np.trunc(a.astype(np.float64) * float(s))
            if r.size == 0 or np.abs(r).max() < 2.0 ** 63:
                return r.astype(np.int64)
            out = np.empty(r.size, dtype=object)
            out[:] = [int(v) for v in r.reshape(-1)]
            return out.reshape(r.shape)
        v = _as_values(a)
        if v.dtype != object and (v.size == 0 or int(np.abs(v).max()) <= _I64_MAX // s):
            return v * s
        return _as_values(np.array([int(x) * s for x in v.reshape(-1)], dtype=object).reshape(v.shape))

    def decode(self, values):
        v = _as_values(values)
        s = self.scale
        if v.dtype != object:
            q = np.abs(v) // s
            return np.where(v < 0, -q, q)
        out = np.empty(v.size, dtype=object)
        out[:] = [(-1 if x < 0 else 1) * (abs(int(x)) // s) for x in v.reshape(-1)]
        return out.reshape(v.shape)


class FloatEncoder(IntegerEncoder):
    """pylib FloatEncoder over the same PlainEncoder (default scale 10^6):
    decode = the value as a double / scale."""

    def __init__(self, scale=10 ** 6):
        super().__init__(scale)

    def decode(self, values):
        v = _as_values(values)
        if v.dtype != object:
            return v.astype(np.float64) / self.scale
        return np.array([float(int(x)) / self.scale for x in v.reshape(-1)], dtype=np.float64).reshape(v.shape)


class BatchEncoder:
    """Two integers per plaintext (phe/encoding/batch_encoder.h:27-140):
    plaintext = (second << (64 + padding_bits)) | first, each value scaled and
    taken as its 64-bit two's-complement bit pattern; padding bits absorb the
    carries of additions.  Packing and unpacking work on limb arrays (NumPy,
    no per-element Python integers), so a packed vector costs one ciphertext
    per pair of values."""

    def __init__(self, scale=1, padding_bits=32):
        if padding_bits < 0:
            raise ValueError("padding_bits must be >= 0")
        self.scale = int(scale)
        self.padding_bits = int(padding_bits)

    def _limbs_needed(self):
        return (128 + self.padding_bits + 31) // 32

    def _aligned(self):
        if self.padding_bits % 32:
            raise ValueError("host packing needs padding_bits a multiple of 32 (the device codec takes any)")

    def pack(self, first, second, pt_limbs):
        """int64 arrays -> (count, pt_limbs) uint32 magnitudes (host form of
        the device codec HG_CODEC_BATCH_I64)."""
        self._aligned()
        a = (np.asarray(first, dtype=np.int64) * self.scale).astype(np.int64).view(np.uint64)
        b = (np.asarray(second, dtype=np.int64) * self.scale).astype(np.int64).view(np.uint64)
        if a.shape != b.shape:
            raise ValueError("first and second must have the same shape")
        need = self._limbs_needed()
        if need > pt_limbs:
            raise ValueError("key too small for this padding")
        out = np.zeros((a.size, pt_limbs), dtype=np.uint32)
        out[:, 0] = (a.reshape(-1) & 0xFFFFFFFF).astype(np.uint32)
        out[:, 1] = (a.reshape(-1) >> np.uint64(32)).astype(np.uint32)
        off = (64 + self.padding_bits) // 32
        out[:, off] = (b.reshape(-1) & 0xFFFFFFFF).astype(np.uint32)
        out[:, off + 1] = (b.reshape(-1) >> np.uint64(32)).astype(np.uint32)
        return out

    def unpack(self, mags, index):
        """(count, pt_limbs) magnitudes -> int64 values of slot `index` (0 or 1)
        divided by the scale (Decode, batch_encoder.h:85-103)."""
        if index not in (0, 1):
            raise ValueError("You cannot get more than two elements from one plaintext")
        self._aligned()
        off = index * ((64 + self.padding_bits) // 32)
        lo = mags[:, off].astype(np.uint64)
        hi = mags[:, off + 1].astype(np.uint64)
        v = (lo | (hi << np.uint64(32))).view(np.int64)
        if self.scale == 1:
            return v
        q = np.abs(v) // self.scale  # C++ division truncates toward zero
        return np.where(v < 0, -q, q)



SCHEMAS = ("zpaillier", "ou")


def setup(key_size=2048, seed=None, device=0, table_window=0, context=None, schema="zpaillier", secret_key=None):
    """Key generation (paillier_z/key_generator.cc:26-60 or
    ou/key_generator.cc:26-96, seeded xoshiro256** stream; a random seed when
    none is given) and engine key load -> HeKit.  ``schema`` names the scheme
    the way heu.phe.setup's SchemaType does (ZPaillier or OU).

    ``setup(public_key)`` with another kit's ``public_key`` dict (or its
    ``public_key_bytes()``, HEU's key wire format) instead of a key size gives
    a kit without the secret key, as heu.phe.setup(pk) does for the side that
    only encrypts and evaluates; ``secret_key=`` (a ``secret_key`` dict or
    ``secret_key_bytes()``) makes it a full kit, as setup(pk, sk) does
    (pylib/phe_binding bind_phe.cc setup overloads)."""
    if isinstance(key_size, (dict, bytes, bytearray)):
        return _setup_public(key_size, device, table_window, context, secret_key)
    schema = schema.lower()
    if schema not in SCHEMAS:
        raise ValueError(f"schema must be one of {SCHEMAS}")
    if seed is None:
        seed = int.from_bytes(os.urandom(8), "little")
    ctx = context or engine.Context(device)
    if schema == "ou":
        k = engine.ou_keygen(key_size, seed)
        key = ctx.load_ou_key(key_size, k["n"], k["G"], k["H"], k["max_pt_bits"], k["p"], k["q"], k["t"],
                              k["gp_inv"], table_window=table_window)
    else:
        k = engine.keygen(key_size, seed)
        key = ctx.load_key(key_size, k["n"], k["h_s"], k["p"], k["q"], table_window=table_window)
    return HeKit(ctx, key, dict(k, key_bits=key_size), schema)


def _setup_public(pk, device, table_window, context, sk=None):
    if isinstance(pk, (bytes, bytearray)):
        _, pk = keywire.deserialize_public_key(pk)
    if isinstance(sk, (bytes, bytearray)):
        _, sk = keywire.deserialize_secret_key(sk)
    schema = "ou" if "G" in pk else "zpaillier"
    n = int(pk["n"])
    if sk is not None and int(sk.get("n", n)) != n:
        raise ValueError("pk and sk are not paired")
    # a k-bit key has an n of k bits (ZPaillier) or a few bits more (OU, ou/key_generator.cc:30-52)
    bits = int(pk.get("key_bits") or (n.bit_length() // 1024) * 1024)
    ctx = context or engine.Context(device)
    sec = {k: int(v) for k, v in (sk or {}).items() if k != "n"}
    if schema == "ou":
        key = ctx.load_ou_key(bits, n, int(pk["G"]), int(pk["H"]), int(pk["max_pt_bits"]), sec.get("p"),
                              sec.get("q"), sec.get("t"), sec.get("gp_inv"), table_window=table_window)
    else:
        key = ctx.load_key(bits, n, int(pk["h_s"]), sec.get("p"), sec.get("q"), table_window=table_window)
    return HeKit(ctx, key, dict(pk, key_bits=bits, **sec), schema)


# Live kits by key, so that unpickled ciphertext arrays find an engine key
# for their n (the pickle holds the wire bytes, not a device handle).
_KITS = weakref.WeakValueDictionary()


def _kit_for(n):
    kits = [k for k in list(_KITS.values()) if k.n == n]
    with_secret = [k for k in kits if k.secret_key is not None]
    return (with_secret or kits or [None])[-1]


def _unpickle_ciphertexts(buf, n):
    kit = _kit_for(n)
    if kit is None:
        raise ValueError("no HeKit for this public key in this process: call hnp.setup(public_key) first")
    return CiphertextArray.load_from(buf, kit)


class HeKit:
    """Key material and engine key of one scheme.  ``max_plaintext`` is the
    bound on |m| that Encrypt checks: n/2 for ZPaillier
    (paillier_z/public_key.h PlaintextBound), 2^(|p/2|-1) for OU
    (ou/key_generator.cc:89-92).  ``random_bits`` is the exact bit length of
    the encryption randomness r, or None where r is any value below 2^(32*r_limbs)."""

    def __init__(self, ctx, key, key_ints, schema="zpaillier"):
        self.context = ctx
        self.key = key
        self.schema = schema
        self.n = key_ints["n"]
        if schema == "ou":
            pub, sec = ("n", "G", "H", "max_pt_bits", "key_bits"), ("p", "q", "t", "gp_inv")
            self.max_plaintext = 1 << key_ints["max_pt_bits"]
            self.random_bits = engine.ou_random_bits(self.n.bit_length())
        else:
            pub, sec = ("n", "h_s", "key_bits"), ("p", "q")
            self.max_plaintext = self.n // 2
            self.random_bits = None
        self.public_key = {k: key_ints[k] for k in pub if k in key_ints}
        has_secret = all(key_ints.get(k) is not None for k in sec)
        self.secret_key = {k: key_ints[k] for k in sec} if has_secret else None
        _KITS[id(self)] = self

    def public_key_bytes(self):
        """PublicKey::Serialize with the schema value (HEU's key wire format)."""
        return keywire.serialize_public_key(self.public_key, self.schema)

    def secret_key_bytes(self):
        if self.secret_key is None:
            raise ValueError("this HeKit was set up from a public key and holds no secret key")
        return keywire.serialize_secret_key(self.secret_key, self.n, self.schema)

    def array(self, values, encoder=None):
        """hnp.array(ndarray, encoder): values encoded by ``encoder`` when one
        is given (integers as they are otherwise)."""
        if encoder is not None and type(encoder) in (IntegerEncoder, FloatEncoder):
            return EncodedArray(values, encoder)
        return PlaintextArray(encoder.encode(values) if encoder is not None else values)

    def integer_encoder(self, scale=1):
        return IntegerEncoder(scale)

    def float_encoder(self, scale=10 ** 6):
        return FloatEncoder(scale)

    def encryptor(self, r_source=None):
        return Encryptor(self, r_source)

    def decryptor(self):
        if self.secret_key is None:
            raise ValueError("this HeKit was set up from a public key and cannot decrypt")
        return Decryptor(self)

    def evaluator(self):
        return Evaluator(self)

    def batch_encoder(self, scale=1, padding_bits=32):
        return BatchEncoder(scale, padding_bits)


class Encryptor:
    """Encrypt(PMatrix) (numpy/encryptor.cc:19-66).  r (k/2 bits,
    encryptor.cc:27) comes from os.urandom, or from ``r_source(count)``
    returning a (count, r_limbs) uint32 array when one is given."""

    def __init__(self, kit, r_source=None):
        self.kit = kit
        self.r_source = r_source

    def _r(self, count):
        key = self.kit.key
        if self.r_source is not None:
            return np.ascontiguousarray(self.r_source(count), dtype=np.uint32).reshape(count, key.r_limbs)
        r = np.frombuffer(os.urandom(count * key.r_limbs * 4), dtype=np.uint32).reshape(count, key.r_limbs).copy()
        bits = self.kit.random_bits
        if bits is not None:  # RandomExactBits(bits): top bit set, nothing above it
            top, off = divmod(bits - 1, 32)
            r[:, top] &= np.uint32((1 << off) - 1)
            r[:, top] |= np.uint32(1 << off)
            r[:, top + 1:] = 0
        return r

    def encrypt(self, pt):
        return self._encrypt(pt)[0]

    def _encrypt(self, pt):
        pt = pt if isinstance(pt, PlaintextArray) else PlaintextArray(pt)
        key = self.kit.key
        dc = pt.device_codec() if isinstance(pt, EncodedArray) and self.kit.schema == "zpaillier" else None
        if dc is not None:
            codec, raw = dc
            r = self._r(raw.size)
            limbs = key.encrypt_encoded(codec, pt.encoder.scale, raw.reshape(-1), r)
            return CiphertextArray(self.kit, limbs, pt.shape), pt, r
        flat = pt.values.reshape(-1)
        r = self._r(flat.size)
        if flat.dtype == object:
            bound = self.kit.max_plaintext
            if any(abs(int(v)) > bound for v in flat):
                raise ValueError("message number out of range")
            limbs = key.encrypt_bn([int(v) for v in flat], r)
        else:
            limbs = key.encrypt(flat, r)
        return CiphertextArray(self.kit, limbs, pt.shape), pt, r

    def encrypt_with_audit(self, pt):
        """EncryptWithAudit (numpy/encryptor.cc:69-104 over
        paillier_zahlen/encryptor.cc:35-65, ou/encryptor.cc:106-136): the
        ciphertexts and, per element, "p:<m>,rn:<h_s^r>,c:<c>" (ZPaillier) or
        "p:<m>,hr:<H^r>,c:<c>" (OU), upper-case hex of the Montgomery-form
        values as BigInt::ToHexString writes them."""
        ct, pt, r = self._encrypt(pt)
        rn = self.kit.key.encrypt_zero(r)
        tag = "hr" if self.kit.schema == "ou" else "rn"
        ints = engine.limbs_to_ints
        audit = [f"p:{_hex(int(m))},{tag}:{_hex(a)},c:{_hex(c)}"
                 for m, a, c in zip(pt.values.reshape(-1), ints(rn), ints(ct.limbs))]
        out = np.empty(len(audit), dtype=object)
        out[:] = audit
        return ct, out.reshape(pt.shape)

    def encrypt_zero(self, shape=()):
        count = int(np.prod(shape, dtype=np.int64))
        return CiphertextArray(self.kit, self.kit.key.encrypt_zero(self._r(count)), shape)

    def encrypt_batch(self, first, second, encoder):
        """Encrypt pairs packed by a BatchEncoder -> CiphertextArray of first's
        shape; ZPaillier keys pack on the device (HG_CODEC_BATCH_I64 / _F64)."""
        key = self.kit.key
        a, b = np.asarray(first), np.asarray(second)
        if a.shape != b.shape:
            raise ValueError("first and second must have the same shape")
        if self.kit.schema == "zpaillier":
            f64 = a.dtype.kind == "f" or b.dtype.kind == "f"
            codec = engine.capi.HG_CODEC_BATCH_F64 if f64 else engine.capi.HG_CODEC_BATCH_I64
            r = self._r(a.size)
            out = key.encrypt_encoded(codec, encoder.scale, a.reshape(-1), r, values2=b.reshape(-1),
                                      padding_bits=encoder.padding_bits)
            return CiphertextArray(self.kit, out, a.shape)
        mags = encoder.pack(first, second, key.pt_limbs)
        neg = np.zeros(mags.shape[0], dtype=np.uint8)
        r = self._r(mags.shape[0])
        out = np.empty((mags.shape[0], key.ct_limbs), dtype=np.uint32)
        engine.capi.check(key.lib.hg_encrypt_bn(key.ctx.handle, key.id, engine._ptr(mags), engine._ptr(neg),
                                                engine._ptr(r), engine._ptr(out), mags.shape[0]))
        return CiphertextArray(self.kit, out, np.asarray(first).shape)


class Decryptor:
    """Decrypt / DecryptInRange (numpy/decryptor.cc:19-99)."""

    def __init__(self, kit):
        self.kit = kit

    def decrypt(self, ct):
        """Decrypt (numpy/decryptor.cc:19-66): the plaintexts, decrypted on
        first use; to_numpy(encoder) on the result decodes on the device."""
        return DecryptedArray(self, ct)

    def _decrypt_values(self, ct):
        key = self.kit.key
        m, ovf = key.decrypt(ct.limbs)
        if ovf.any():
            vals = np.empty(ct.size, dtype=object)
            vals[:] = key.decrypt_bn(ct.limbs)
            return _as_values(vals.reshape(ct.shape))
        return _as_values(m.reshape(ct.shape))

    def decrypt_batch(self, ct, encoder, as_float=False):
        """Decrypt packed ciphertexts -> (first, second) int64 arrays (float64
        with as_float, BatchEncoder::Decode<double>); ZPaillier keys unpack
        on the device."""
        key = self.kit.key
        if self.kit.schema == "zpaillier":
            codec = engine.capi.HG_CODEC_BATCH_F64 if as_float else engine.capi.HG_CODEC_BATCH_I64
            s0, s1, neg = key.decrypt_decoded(codec, encoder.scale, ct.limbs, padding_bits=encoder.padding_bits)
            if neg.any():
                raise ValueError("packed plaintext is negative: a slot underflowed its padding")
            return s0.reshape(ct.shape), s1.reshape(ct.shape)
        mag = np.empty((ct.size, key.pt_limbs), dtype=np.uint32)
        neg = np.empty(ct.size, dtype=np.uint8)
        engine.capi.check(key.lib.hg_decrypt_bn(key.ctx.handle, key.id, engine._ptr(ct.limbs), engine._ptr(mag),
                                                engine._ptr(neg), ct.size))
        if neg.any():
            raise ValueError("packed plaintext is negative: a slot underflowed its padding")
        return encoder.unpack(mag, 0).reshape(ct.shape), encoder.unpack(mag, 1).reshape(ct.shape)

    def decrypt_in_range(self, ct, range_bits=128):
        vals = self.kit.key.decrypt_in_range(ct.limbs, range_bits)
        if isinstance(vals, list):
            out = np.empty(len(vals), dtype=object)
            out[:] = vals
            return PlaintextArray(out.reshape(ct.shape))
        return PlaintextArray(np.asarray(vals).reshape(ct.shape))


def _broadcast_index(shape_x, shape_y):
    try:
        out = np.broadcast_shapes(shape_x, shape_y)
    except ValueError:
        raise ValueError(f"operands could not be broadcast together: dim(x)={shape_x}, dim(y)={shape_y}")
    ix = np.broadcast_to(np.arange(int(np.prod(shape_x, dtype=np.int64))).reshape(shape_x), out).reshape(-1)
    iy = np.broadcast_to(np.arange(int(np.prod(shape_y, dtype=np.int64))).reshape(shape_y), out).reshape(-1)
    return out, ix, iy


class Evaluator:
    """heu.numpy Evaluator (numpy/evaluator.h:23-87) on the engine."""

    def __init__(self, kit):
        self.kit = kit
        self.key = kit.key

    # -- element-wise ------------------------------------------------------
    def _plain_i64(self, p, idx):
        v = p.values.reshape(-1)[idx]
        if v.dtype == object:
            return None, v
        return np.ascontiguousarray(v, dtype=np.int64), None

    def add(self, x, y):
        if isinstance(x, PlaintextArray) and isinstance(y, PlaintextArray):
            return PlaintextArray(_as_values(x.values.astype(object) + y.values.astype(object)))
        if isinstance(x, PlaintextArray):
            x, y = y, x
        shape, ix, iy = _broadcast_index(x.shape, y.shape)
        a = x.limbs[ix]
        if isinstance(y, CiphertextArray):
            return CiphertextArray(self.kit, self.key.add(a, y.limbs[iy]), shape)
        p64, big = self._plain_i64(y, iy)
        if p64 is not None:
            return CiphertextArray(self.kit, self.key.add_plain(a, p64), shape)
        # full-range addends: (1 + p*n) is the encryption of p with r = 0
        g = self.key.encrypt_bn([int(v) for v in big], np.zeros((len(big), self.key.r_limbs), np.uint32))
        return CiphertextArray(self.kit, self.key.add(a, g), shape)

    def sub(self, x, y):
        """Sub (numpy/evaluator.cc:160-185 over evaluator.cc:66-84)."""
        if isinstance(x, PlaintextArray) and isinstance(y, PlaintextArray):
            return PlaintextArray(_as_values(x.values.astype(object) - y.values.astype(object)))
        if isinstance(y, PlaintextArray):
            return self.add(x, PlaintextArray(_as_values(-y.values.astype(object))))
        shape, ix, iy = _broadcast_index(x.shape, y.shape)
        if isinstance(x, CiphertextArray):
            return CiphertextArray(self.kit, self.key.sub(x.limbs[ix], y.limbs[iy]), shape)
        neg = CiphertextArray(self.kit, self.key.negate(y.limbs[iy]), shape)
        return self.add(neg, PlaintextArray(x.values.reshape(-1)[ix].reshape(shape)))

    def mul(self, x, y):
        if isinstance(x, PlaintextArray) and isinstance(y, PlaintextArray):
            return PlaintextArray(_as_values(x.values.astype(object) * y.values.astype(object)))
        if isinstance(x, PlaintextArray):
            x, y = y, x
        if not isinstance(y, PlaintextArray):
            raise TypeError("ciphertext * ciphertext is not defined for Paillier")
        shape, ix, iy = _broadcast_index(x.shape, y.shape)
        p64, big = self._plain_i64(y, iy)
        if p64 is None:
            # scalars of any size (evaluator.cc:99-123 takes any BigInt)
            return CiphertextArray(self.kit, self.key.mul_bn(x.limbs[ix], [int(v) for v in big]), shape)
        return CiphertextArray(self.kit, self.key.mul(x.limbs[ix], p64), shape)

    def negate(self, x):
        return CiphertextArray(self.kit, self.key.negate(x.limbs), x.shape)

    def randomize(self, x, r=None):
        r = r if r is not None else Encryptor(self.kit)._r(x.size)
        return CiphertextArray(self.kit, self.key.randomize(x.limbs, r), x.shape)

    # -- reductions --------------------------------------------------------
    def sum(self, x):
        """Sum of all elements (numpy/evaluator.cc:355-373)."""
        if isinstance(x, PlaintextArray):
            return int(np.sum(x.values.astype(object)))
        if x.size == 0:
            raise ValueError("you cannot sum an empty tensor")
        return CiphertextArray(self.kit, self.key.sum(x.limbs), ())

    def select_sum(self, x, item):
        """Sum of x[item] (extension_functions.cc:28-58)."""
        if isinstance(x, PlaintextArray):
            return int(np.sum(np.asarray(x.values[item]).astype(object)))
        if x.size == 0:
            raise ValueError(f"you cannot select sum an empty tensor, shape={x.shape}")
        sub = x[item]
        if sub.size == 0:
            return CiphertextArray(self.kit, self.key._identity(), ())
        return CiphertextArray(self.kit, self.key.sum(sub.limbs), ())

    def batch_select_sum(self, x, items):
        """[select_sum(x, it) for it in items] (extension_functions.cc:60-78),
        grouped into bucket-sum launches of up to 256 selections."""
        if isinstance(x, PlaintextArray):
            return PlaintextArray(_as_values([self.select_sum(x, it) for it in items]))
        if x.size == 0:
            raise ValueError(f"you cannot select sum an empty tensor, shape={x.shape}")
        idx = np.arange(x.size).reshape(x.shape)
        sels = [np.asarray(idx[it]).reshape(-1) for it in items]
        out = self.key.batch_select_sum(x.limbs, sels)
        return CiphertextArray(self.kit, out, (len(items),))

    def feature_wise_bucket_sum(self, x, subgroup_map, order_map, bucket_num, cumsum=False):
        """FeatureWiseBucketSum over the rows selected by subgroup_map
        (extension_functions.cc:89-107; numpy/evaluator.cc:378-458).
        Returns (bucket_num * features, cols)."""
        rows = np.nonzero(np.asarray(subgroup_map).reshape(-1) > 0)[0]
        om = np.asarray(order_map)
        grid = x.grid() if x.ndim == 2 else x.grid().reshape(x.shape[0], 1, -1)
        feats = om.shape[1]
        cols = grid.shape[1]
        if len(rows) == 0:
            zero = self.key._identity()
            return CiphertextArray(self.kit, np.repeat(zero, bucket_num * feats * cols, axis=0),
                                   (bucket_num * feats, cols))
        out = self.key.bucket_sum(grid[rows], om[rows].astype(np.uint8), bucket_num, cumsum=cumsum)
        return CiphertextArray(self.kit, out.reshape(-1, self.key.ct_limbs), (bucket_num * feats, cols))

    def batch_feature_wise_bucket_sum(self, x, subgroup_maps, order_map, bucket_num, cumsum=False):
        """One feature_wise_bucket_sum per subgroup map (extension_functions.cc:109-138)."""
        return [self.feature_wise_bucket_sum(x, sm, order_map, bucket_num, cumsum) for sm in subgroup_maps]

    def matmul(self, x, y):
        """MatMul (numpy/evaluator.cc:208-353): ciphertext @ plaintext or
        plaintext @ ciphertext, with NumPy's 1-D rules ((K,) @ (K, N) -> (N,),
        (M, K) @ (K,) -> (M,))."""
        if isinstance(x, CiphertextArray) and isinstance(y, PlaintextArray):
            xv = x.grid() if x.ndim == 2 else x.grid().reshape(1, x.shape[0], -1)
            yv = _matmul_plain(y.values)
            yv = yv if yv.ndim == 2 else yv.reshape(-1, 1)
            out = self.key.matmul(xv, yv)
        elif isinstance(x, PlaintextArray) and isinstance(y, CiphertextArray):
            # (P @ C)^T = C^T @ P^T
            yv = y.grid() if y.ndim == 2 else y.grid().reshape(y.shape[0], 1, -1)
            ct_t = np.ascontiguousarray(np.transpose(yv, (1, 0, 2)))
            pv = _matmul_plain(x.values)
            pv = pv if pv.ndim == 2 else pv.reshape(1, -1)
            out = np.ascontiguousarray(np.transpose(self.key.matmul(ct_t, np.ascontiguousarray(pv.T)), (1, 0, 2)))
        else:
            raise TypeError("matmul needs one ciphertext and one plaintext operand")
        shape = out.shape[:2]
        if x.ndim == 1:
            shape = shape[1:]
        if y.ndim == 1:
            shape = shape[:-1]
        return CiphertextArray(self.kit, out.reshape(-1, self.key.ct_limbs), shape)

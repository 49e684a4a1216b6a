"""Python host layer over the C-ABI: contexts, keys and batched operations on
NumPy arrays.

Names follow HEU's phe / heu.numpy interfaces for the ZPaillier path
(heu/library/phe/encryptor.h, decryptor.h, evaluator.h; heu/library/numpy/
evaluator.h): a loaded key exposes encrypt / decrypt / add / sub / mul /
negate / randomize / sum over batches.  Ciphertexts are uint32 arrays of
shape (count, S) in Montgomery form (HEU's in-memory representation);
``from_mont`` gives the canonical Z-form.
"""

import ctypes

import numpy as np

from heu_gb300 import capi


def ints_to_limbs(values, nlimbs):
    """Non-negative Python ints -> uint32 array (count, nlimbs), little-endian."""
    nb = 4 * nlimbs
    buf = b"".join(int(v).to_bytes(nb, "little") for v in values)
    return np.frombuffer(buf, dtype="<u4").reshape(len(values), nlimbs).copy()


def limbs_to_ints(arr):
    arr = np.ascontiguousarray(arr, dtype="<u4")
    if arr.ndim == 1:
        arr = arr.reshape(1, -1)
    raw = arr.tobytes()
    nb = arr.shape[1] * 4
    return [int.from_bytes(raw[i * nb:(i + 1) * nb], "little") for i in range(arr.shape[0])]


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _u32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    if shape is not None and a.shape != shape:
        a = a.reshape(shape)
    return a


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64).reshape(-1)


def keygen(key_bits, seed):
    """key_generator.cc:26-60 from a seeded stream -> dict of ints n, p, q, h_s."""
    lib = capi.load()
    n = np.zeros(key_bits // 32, np.uint32)
    p = np.zeros(key_bits // 64, np.uint32)
    q = np.zeros(key_bits // 64, np.uint32)
    hs = np.zeros(key_bits // 16, np.uint32)
    capi.check(lib.hg_keygen(key_bits, seed & (2 ** 64 - 1), _ptr(n), _ptr(p), _ptr(q), _ptr(hs)))
    return {
        "n": limbs_to_ints(n)[0],
        "p": limbs_to_ints(p)[0],
        "q": limbs_to_ints(q)[0],
        "h_s": limbs_to_ints(hs)[0],
    }


def backend_radix_bits(n2_bits, backend):
    """Montgomery radix exponent of a yacl BigInt backend for a modulus of
    n2_bits bits: OpenSSL's BN_MONT_CTX and GMP use 64-bit limbs (R =
    2^(64 * ceil(bits / 64))), libtommath 60-bit digits (R = 2^(60 *
    ceil(bits / 60)))."""
    if backend in ("openssl", "gmp"):
        return 64 * -(-n2_bits // 64)
    if backend == "tommath":
        return 60 * -(-n2_bits // 60)
    raise ValueError("backend must be openssl, gmp or tommath")


def radix_constant(n2, limbs, radix_bits, to_external):
    """The constant C with MM(c * R, C) = c * R_ext (to_external) or
    MM(c * R_ext, C) = c * R mod n2, R = 2^(32 * limbs), R_ext = 2^radix_bits,
    MM(x, y) = x * y * R^-1 mod n2."""
    r_in = pow(2, 32 * limbs, n2)
    r_ext = pow(2, radix_bits, n2)
    if to_external:
        return r_ext  # MM(c R, R_ext) = c R_ext
    return r_in * r_in * pow(r_ext, -1, n2) % n2  # MM(c R_ext, R^2 / R_ext) = c R


def ou_sizes(key_bits):
    """(ciphertext limbs S, secret limbs S/2) of an OU key."""
    if key_bits == 1024:
        return 64, 32
    if key_bits in (2048, 3072):
        return 128, 64
    raise ValueError("OU keys of 1024, 2048 or 3072 bits")


def matrix_dims(shape):
    """NumPy shape -> (rows, cols, ndim) of heu.numpy's DenseMatrix: a scalar
    is 1 x 1, a vector n x 1 (numpy/shape.h:44-54)."""
    if len(shape) == 0:
        return 1, 1, 0
    if len(shape) == 1:
        return int(shape[0]), 1, 1
    if len(shape) == 2:
        return int(shape[0]), int(shape[1]), 2
    raise ValueError("HEU tensor dimension cannot exceed 2")


def numpy_shape(rows, cols, ndim):
    return () if ndim == 0 else (rows,) if ndim == 1 else (rows, cols)


def ou_random_bits(n_bits):
    """Bit length of OU encryption randomness for an n of n_bits bits
    (ou/encryptor.cc:12-20 with ou/public_key.h:27-31): 80 / 110 / 128."""
    if n_bits >= 2560:
        return 128
    if n_bits >= 1536:
        return 110
    return 80


def ou_keygen(key_bits, seed):
    """ou/key_generator.cc:26-96 from a seeded stream -> dict of ints n, G, H,
    p, q, t, gp_inv and max_pt_bits."""
    lib = capi.load()
    S, H = ou_sizes(key_bits)
    bufs = {k: np.zeros(S if k in ("n", "G", "H") else H, np.uint32) for k in ("n", "G", "H", "p", "q", "t", "gp_inv")}
    mb = ctypes.c_int()
    capi.check(lib.hg_ou_keygen(key_bits, seed & (2 ** 64 - 1), *[_ptr(bufs[k]) for k in ("n", "G", "H", "p", "q", "t",
                                                                                        "gp_inv")],
                                ctypes.byref(mb)))
    out = {k: limbs_to_ints(v)[0] for k, v in bufs.items()}
    out["max_pt_bits"] = mb.value
    return out


class Context:
    """One engine context on one device (hg_ctx)."""

    def __init__(self, device=0):
        self.lib = capi.load()
        h = ctypes.c_void_p()
        capi.check(self.lib.hg_ctx_create(device, ctypes.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            self.lib.hg_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sm_count(self):
        return self.lib.hg_device_sm_count(self.handle)

    def load_ou_key(self, key_bits, n, G, H, max_pt_bits, p=None, q=None, t=None, gp_inv=None, table_window=0):
        """An Okamoto-Uchiyama key (ou/public_key.cc, secret_key.h) -> Key."""
        S, Hh = ou_sizes(key_bits)
        # keep every limb array alive until the call returns
        arrs = [ints_to_limbs([v], k) if v is not None else None
                for v, k in ((n, S), (G, S), (H, S), (p, Hh), (q, Hh), (t, Hh), (gp_inv, Hh))]
        kid = ctypes.c_int()
        capi.check(self.lib.hg_ou_key_load(self.handle, key_bits, _ptr(arrs[0]), _ptr(arrs[1]), _ptr(arrs[2]),
                                           max_pt_bits, _ptr(arrs[3]), _ptr(arrs[4]), _ptr(arrs[5]), _ptr(arrs[6]),
                                           table_window, ctypes.byref(kid)))
        return Key(self, kid.value, key_bits, n)

    def load_key(self, key_bits, n, h_s, p=None, q=None, table_window=0):
        S = key_bits // 16
        n_l = ints_to_limbs([n], S // 2)
        hs_l = ints_to_limbs([h_s], S)
        p_l = ints_to_limbs([p], S // 4) if p is not None else None
        q_l = ints_to_limbs([q], S // 4) if q is not None else None
        kid = ctypes.c_int()
        capi.check(self.lib.hg_key_load(self.handle, key_bits, _ptr(n_l), _ptr(hs_l), _ptr(p_l), _ptr(q_l),
                                        table_window, ctypes.byref(kid)))
        return Key(self, kid.value, key_bits, n)


class Key:
    def __init__(self, ctx, key_id, key_bits, n):
        self.ctx = ctx
        self.lib = ctx.lib
        self.id = key_id
        self.key_bits = key_bits
        self.n = n
        s, r, pl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        capi.check(self.lib.hg_key_shape(ctx.handle, key_id, ctypes.byref(s), ctypes.byref(r), ctypes.byref(pl)))
        self.ct_limbs, self.r_limbs, self.pt_limbs = s.value, r.value, pl.value

    # -- helpers ----------------------------------------------------------
    def _ct(self, a):
        a = np.ascontiguousarray(a, dtype=np.uint32)
        return a.reshape(-1, self.ct_limbs)

    def _out(self, count):
        return np.empty((count, self.ct_limbs), dtype=np.uint32)

    def free(self):
        capi.check(self.lib.hg_key_free(self.ctx.handle, self.id))

    # -- encryption -------------------------------------------------------
    def encrypt(self, m, r):
        m = _i64(m)
        r = _u32(r).reshape(-1, self.r_limbs)
        out = self._out(m.size)
        capi.check(self.lib.hg_encrypt(self.ctx.handle, self.id, _ptr(m), _ptr(r), _ptr(out), m.size))
        return out

    def encrypt_bn(self, ms, r):
        mags = ints_to_limbs([abs(int(v)) for v in ms], self.pt_limbs)
        neg = np.array([1 if int(v) < 0 else 0 for v in ms], dtype=np.uint8)
        r = _u32(r).reshape(-1, self.r_limbs)
        out = self._out(len(ms))
        capi.check(self.lib.hg_encrypt_bn(self.ctx.handle, self.id, _ptr(mags), _ptr(neg), _ptr(r), _ptr(out),
                                          len(ms)))
        return out

    def encrypt_encoded(self, codec, scale, values, r, values2=None, padding_bits=32):
        """Encrypt raw int64 / double values encoded on the device (HG_CODEC_*:
        PlainEncoder, plain_encoder.h:46-74; BatchEncoder, batch_encoder.h:
        27-140, with values2 as the second slot)."""
        f64 = codec in (capi.HG_CODEC_PLAIN_F64, capi.HG_CODEC_BATCH_F64)
        dt = np.float64 if f64 else np.int64
        v = np.ascontiguousarray(values, dtype=dt).reshape(-1)
        v2 = None if values2 is None else np.ascontiguousarray(values2, dtype=dt).reshape(-1)
        if v2 is not None and v2.size != v.size:
            raise ValueError("both slots need the same number of values")
        r = _u32(r).reshape(-1, self.r_limbs)
        out = self._out(v.size)
        capi.check(self.lib.hg_encrypt_encoded(self.ctx.handle, self.id, codec, int(scale), int(padding_bits), _ptr(v),
                                               _ptr(v2), _ptr(r), _ptr(out), v.size))
        return out

    def decrypt_decoded(self, codec, scale, ct, padding_bits=32):
        """Decrypt and decode on the device -> (values, overflow) or, for the
        batch codecs, (slot0, slot1, overflow)."""
        ct = self._ct(ct)
        n = ct.shape[0]
        f64 = codec in (capi.HG_CODEC_PLAIN_F64, capi.HG_CODEC_BATCH_F64)
        dt = np.float64 if f64 else np.int64
        out = np.empty(n, dtype=dt)
        batch = codec in (capi.HG_CODEC_BATCH_I64, capi.HG_CODEC_BATCH_F64)
        out2 = np.empty(n, dtype=dt) if batch else None
        ovf = np.empty(n, dtype=np.uint8)
        capi.check(self.lib.hg_decrypt_decoded(self.ctx.handle, self.id, codec, int(scale), int(padding_bits),
                                               _ptr(ct), _ptr(out), _ptr(out2), _ptr(ovf), n))
        return (out, out2, ovf) if batch else (out, ovf)

    def convert_radix(self, ct, radix_bits, to_external):
        """c * R <-> c * 2^radix_bits mod n^2 (hg_convert_radix)."""
        ct = self._ct(ct)
        out = self._out(ct.shape[0])
        capi.check(self.lib.hg_convert_radix(self.ctx.handle, self.id, _ptr(ct), _ptr(out), ct.shape[0],
                                             int(radix_bits), 1 if to_external else 0))
        return out

    def encrypt_zero(self, r):
        r = _u32(r).reshape(-1, self.r_limbs)
        out = self._out(r.shape[0])
        capi.check(self.lib.hg_encrypt_zero(self.ctx.handle, self.id, _ptr(r), _ptr(out), r.shape[0]))
        return out

    def randomize(self, ct, r):
        out = self._ct(ct).copy()
        r = _u32(r).reshape(-1, self.r_limbs)
        capi.check(self.lib.hg_randomize(self.ctx.handle, self.id, _ptr(out), _ptr(r), out.shape[0]))
        return out

    # -- decryption -------------------------------------------------------
    def decrypt(self, ct):
        ct = self._ct(ct)
        m = np.empty(ct.shape[0], dtype=np.int64)
        ovf = np.empty(ct.shape[0], dtype=np.uint8)
        capi.check(self.lib.hg_decrypt(self.ctx.handle, self.id, _ptr(ct), _ptr(m), _ptr(ovf), ct.shape[0]))
        return m, ovf

    def decrypt_bn(self, ct):
        ct = self._ct(ct)
        mag = np.empty((ct.shape[0], self.pt_limbs), dtype=np.uint32)
        neg = np.empty(ct.shape[0], dtype=np.uint8)
        capi.check(self.lib.hg_decrypt_bn(self.ctx.handle, self.id, _ptr(ct), _ptr(mag), _ptr(neg), ct.shape[0]))
        return [(-v if s else v) for v, s in zip(limbs_to_ints(mag), neg)]

    def decrypt_in_range(self, ct, range_bits=64):
        """heu.numpy DecryptInRange (numpy/decryptor.cc:24-47, 86-99): decrypt
        and raise if any plaintext's magnitude has more than `range_bits` bits.
        Returns int64 values when range_bits <= 63, Python ints otherwise."""
        if range_bits <= 63:
            m, ovf = self.decrypt(ct)
            lim = 1 << range_bits  # |m| has more than range_bits bits iff |m| >= lim
            bad = ovf.astype(bool) | (m == np.iinfo(np.int64).min)
            if range_bits < 63:
                bad |= (m >= lim) | (m <= -lim)
            if bad.any():
                i = int(np.nonzero(bad)[0][0])
                found = abs(self.decrypt_bn(self._ct(ct)[i:i + 1])[0]).bit_length()
                raise ValueError("Dangerous!!! HE ciphertext range check failed, there may be a malicious party "
                                 f"stealing your data, please stop computing immediately. found "
                                 f"pt.BitCount()={found}, expected {range_bits}")
            return m
        vals = self.decrypt_bn(ct)
        for v in vals:
            if abs(v).bit_length() > range_bits:
                raise ValueError("Dangerous!!! HE ciphertext range check failed, there may be a malicious party "
                                 f"stealing your data, please stop computing immediately. found "
                                 f"pt.BitCount()={abs(v).bit_length()}, expected {range_bits}")
        return vals

    # -- evaluator --------------------------------------------------------
    def _binary_ct(self, fn, a, b):
        a, b = self._ct(a), self._ct(b)
        if a.shape != b.shape:
            raise ValueError("shape mismatch")
        out = self._out(a.shape[0])
        capi.check(fn(self.ctx.handle, self.id, _ptr(a), _ptr(b), _ptr(out), a.shape[0]))
        return out

    def _ct_pt(self, fn, a, p):
        a, p = self._ct(a), _i64(p)
        if a.shape[0] != p.size:
            raise ValueError("shape mismatch")
        out = self._out(a.shape[0])
        capi.check(fn(self.ctx.handle, self.id, _ptr(a), _ptr(p), _ptr(out), a.shape[0]))
        return out

    def add(self, a, b):
        return self._binary_ct(self.lib.hg_add, a, b)

    def sub(self, a, b):
        return self._binary_ct(self.lib.hg_sub, a, b)

    def add_plain(self, a, p):
        return self._ct_pt(self.lib.hg_add_plain, a, p)

    def sub_plain(self, a, p):
        return self._ct_pt(self.lib.hg_sub_plain, a, p)

    def plain_sub(self, p, a):
        a, p = self._ct(a), _i64(p)
        out = self._out(a.shape[0])
        capi.check(self.lib.hg_plain_sub(self.ctx.handle, self.id, _ptr(p), _ptr(a), _ptr(out), a.shape[0]))
        return out

    def mul(self, a, k):
        """Mul(ct, k) (evaluator.cc:99-123).  k: int64 array, or Python ints of
        any size up to the width of n^2 (then hg_mul_bn)."""
        k_arr = np.asarray(k)
        if k_arr.dtype != object and np.issubdtype(k_arr.dtype, np.integer) and k_arr.dtype.itemsize <= 8 and \
                k_arr.dtype != np.uint64:
            return self._ct_pt(self.lib.hg_mul, a, k_arr)
        ks = [int(v) for v in k_arr.reshape(-1)]
        if all(-(2 ** 63) <= v < 2 ** 63 for v in ks):
            return self._ct_pt(self.lib.hg_mul, a, np.array(ks, dtype=np.int64))
        return self.mul_bn(a, ks)

    def mul_bn(self, a, ks):
        a = self._ct(a)
        ks = [int(v) for v in ks]
        if a.shape[0] != len(ks):
            raise ValueError("shape mismatch")
        width = max(1, max((abs(v).bit_length() + 31) // 32 for v in ks) if ks else 1)
        if width > self.ct_limbs:
            raise ValueError("scalar wider than n^2")
        mags = ints_to_limbs([abs(v) for v in ks], width)
        neg = np.array([1 if v < 0 else 0 for v in ks], dtype=np.uint8)
        out = self._out(a.shape[0])
        capi.check(self.lib.hg_mul_bn(self.ctx.handle, self.id, _ptr(a), _ptr(mags), _ptr(neg), width, _ptr(out),
                                      a.shape[0]))
        return out

    def negate(self, a):
        a = self._ct(a)
        out = self._out(a.shape[0])
        capi.check(self.lib.hg_negate(self.ctx.handle, self.id, _ptr(a), _ptr(out), a.shape[0]))
        return out

    # -- HEU wire format (numpy/matrix.h:221-310) --------------------------
    def serialize(self, ct, shape=None):
        """Ciphertexts in C order with NumPy shape `shape` (default: a vector)
        -> the bytes of DenseMatrix<Ciphertext>::Serialize."""
        ct = self._ct(ct)
        shape = tuple(shape) if shape is not None else (ct.shape[0],)
        rows, cols, ndim = matrix_dims(shape)
        if rows * cols != ct.shape[0]:
            raise ValueError(f"shape {shape} does not hold {ct.shape[0]} ciphertexts")
        bound = ctypes.c_size_t()
        capi.check(self.lib.hg_serialize_bound(self.ctx.handle, self.id, ct.shape[0], ctypes.byref(bound)))
        out = np.empty(max(bound.value, 1), np.uint8)
        n = ctypes.c_size_t()
        capi.check(self.lib.hg_serialize(self.ctx.handle, self.id, _ptr(ct), rows, cols, ndim, 1, _ptr(out), out.size,
                                         ctypes.byref(n)))
        return out[:n.value].tobytes()

    def deserialize(self, buf):
        """DenseMatrix<Ciphertext>::LoadFrom -> (limbs in C order, NumPy shape)."""
        b = np.frombuffer(buf, dtype=np.uint8)
        rows, cols, ndim = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_int()
        args = (self.ctx.handle, self.id, _ptr(b), b.size, 1)
        shp = (ctypes.byref(rows), ctypes.byref(cols), ctypes.byref(ndim))
        rc = self.lib.hg_deserialize(*args, None, 0, *shp)
        if rc != capi.HG_OK and rows.value * cols.value == 0:
            capi.check(rc)
        out = self._out(rows.value * cols.value)
        capi.check(self.lib.hg_deserialize(*args, _ptr(out), out.shape[0], *shp))
        return out, numpy_shape(rows.value, cols.value, ndim.value)

    def sum(self, a):
        a = self._ct(a)
        out = self._out(1)
        capi.check(self.lib.hg_sum(self.ctx.handle, self.id, _ptr(a), a.shape[0], _ptr(out)))
        return out

    def to_mont(self, z):
        z = self._ct(z)
        out = self._out(z.shape[0])
        capi.check(self.lib.hg_to_mont(self.ctx.handle, self.id, _ptr(z), _ptr(out), z.shape[0]))
        return out

    def from_mont(self, m):
        m = self._ct(m)
        out = self._out(m.shape[0])
        capi.check(self.lib.hg_from_mont(self.ctx.handle, self.id, _ptr(m), _ptr(out), m.shape[0]))
        return out

    # -- heu.numpy reductions ----------------------------------------------
    def bucket_sum(self, x, order_map, bucket_num, cumsum=False):
        """FeatureWiseBucketSum: x (rows, cols, S) or (rows, S) ciphertexts,
        order_map (rows, features) uint8 bin ids -> (features*bucket_num, cols, S)."""
        x = np.ascontiguousarray(x, dtype=np.uint32)
        if x.ndim == 2:
            x = x.reshape(x.shape[0], 1, x.shape[1])
        rows, cols = x.shape[0], x.shape[1]
        om = np.ascontiguousarray(order_map, dtype=np.uint8)
        if om.ndim != 2 or om.shape[0] != rows:
            raise ValueError("order map and x should have same number of rows.")
        feats = om.shape[1]
        out = np.empty((feats * bucket_num, cols, self.ct_limbs), dtype=np.uint32)
        capi.check(self.lib.hg_bucket_sum(self.ctx.handle, self.id, _ptr(x), rows, cols, _ptr(om), feats,
                                          bucket_num, 1 if cumsum else 0, _ptr(out)))
        return out

    def matmul(self, x, y):
        """Ciphertext matrix x (M, K, S) times integer matrix y (K, N) -> (M, N, S).
        y: int64, or Python ints of any size up to the width of n^2 (then
        hg_matmul_bn)."""
        x = np.ascontiguousarray(x, dtype=np.uint32)
        y = np.asarray(y)
        M, K = x.shape[0], x.shape[1]
        if y.ndim != 2 or y.shape[0] != K:
            raise ValueError("dimension mismatch for matmul")
        N = y.shape[1]
        out = np.empty((M, N, self.ct_limbs), dtype=np.uint32)
        if y.dtype == object or y.dtype == np.uint64:
            vals = [int(v) for v in y.reshape(-1)]
            if not all(-(2 ** 63) <= v < 2 ** 63 for v in vals):
                width = max(1, max((abs(v).bit_length() + 31) // 32 for v in vals))
                if width > self.ct_limbs:
                    raise ValueError("plaintext wider than n^2")
                mags = ints_to_limbs([abs(v) for v in vals], width)
                neg = np.array([1 if v < 0 else 0 for v in vals], dtype=np.uint8)
                capi.check(self.lib.hg_matmul_bn(self.ctx.handle, self.id, _ptr(x), M, K, _ptr(mags), _ptr(neg), width,
                                                 N, _ptr(out)))
                return out
            y = np.array(vals, dtype=np.int64).reshape(K, N)
        y = np.ascontiguousarray(y, dtype=np.int64)
        capi.check(self.lib.hg_matmul(self.ctx.handle, self.id, _ptr(x), M, K, _ptr(y), N, _ptr(out)))
        return out

    def select_sum(self, x, rows, cols=None):
        """numpy Evaluator::SelectSum (numpy/evaluator.h:57-70) behind the pylib
        select_sum extension (pylib/numpy_binding/extension_functions.cc:28-58):
        the Sum of x[rows] (x of shape (n, S)) or x[rows][:, cols] (x of shape
        (n, m, S)); `rows`/`cols` are anything NumPy indexes with (int arrays,
        lists, slices, masks).  An empty tensor is an error; an empty selection
        gives the ciphertext Sub(x[0], x[0]), the identity."""
        x = np.ascontiguousarray(x, dtype=np.uint32)
        if x.size == 0:
            raise ValueError(f"you cannot select sum an empty tensor, shape={x.shape[:-1]}")
        if x.ndim == 2:
            if cols is not None:
                raise ValueError("too many indices for array")
            sub = x[rows]
        else:
            sub = x[rows][:, cols] if cols is not None else x[rows]
        sub = sub.reshape(-1, self.ct_limbs)
        if sub.shape[0] == 0:
            return self._identity()
        return self.sum(sub)

    def batch_select_sum(self, x, selections):
        """pylib batch_select_sum (extension_functions.cc:60-78): one Sum per row
        selection, as (len(selections), S).  All selections of a group of up to
        256 run as one bucket-sum launch (bucket = selection number) instead
        of one reduction each."""
        x = np.ascontiguousarray(x, dtype=np.uint32)
        if x.size == 0:
            raise ValueError(f"you cannot select sum an empty tensor, shape={x.shape[:-1]}")
        flat = x.reshape(x.shape[0], -1, self.ct_limbs)
        out = np.empty((len(selections), self.ct_limbs), dtype=np.uint32)
        for g0 in range(0, len(selections), 256):
            group = selections[g0:g0 + 256]
            parts, ids = [], []
            for b, sel in enumerate(group):
                sub = flat[sel].reshape(-1, self.ct_limbs)
                parts.append(sub)
                ids.append(np.full(sub.shape[0], b, dtype=np.uint8))
            if sum(p.shape[0] for p in parts) == 0:
                out[g0:g0 + len(group)] = self._identity()
                continue
            xs = np.concatenate(parts, axis=0)
            om = np.concatenate(ids).reshape(-1, 1)
            res = self.bucket_sum(xs, om, len(group))
            out[g0:g0 + len(group)] = res.reshape(len(group), self.ct_limbs)
        return out

    def _identity(self):
        """Montgomery form of 1: Sub(c, c) for any valid c (evaluator.h:84-87)."""
        r = np.zeros((1, self.r_limbs), dtype=np.uint32)
        return self.encrypt(np.zeros(1, dtype=np.int64), r)

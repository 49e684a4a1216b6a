"""ctypes wrapper of the oracle's C restatement (oracle/c/paillier_z_ref.c).

TEST INFRASTRUCTURE ONLY: used by tests/ as a second checker and by the CPU
legs of bench.py as the timed paillier_z baseline.
"""

import ctypes
import os

import numpy as np

from oracle import cbuild
from oracle import paillier_z as pz

_lib = None


def load():
    global _lib
    if _lib is None:
        cbuild.build()
        lib = ctypes.CDLL(cbuild.LIB)
        P = ctypes.c_void_p
        lib.pz_key_create.argtypes = [ctypes.c_int] + [P] * 9 + [ctypes.c_int]
        lib.pz_key_create.restype = P
        lib.pz_key_free.argtypes = [P]
        for name, args in (
            ("pz_encrypt", [P, P, P, P, ctypes.c_size_t, ctypes.c_int]),
            ("pz_decrypt", [P, P, P, P, ctypes.c_size_t, ctypes.c_int]),
            ("pz_add", [P, P, P, P, ctypes.c_size_t, ctypes.c_int]),
            ("pz_mul", [P, P, P, P, ctypes.c_size_t, ctypes.c_int]),
            ("pz_sum", [P, P, ctypes.c_size_t, P]),
            ("pz_sum_mt", [P, P, ctypes.c_size_t, P, ctypes.c_int]),
            ("pz_bucket_sum", [P, P, ctypes.c_size_t, P, ctypes.c_size_t, ctypes.c_size_t, P, ctypes.c_int]),
            ("pz_matmul", [P, P, ctypes.c_size_t, ctypes.c_size_t, P, ctypes.c_size_t, P, ctypes.c_int]),
        ):
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _lib = lib
    return _lib


def _u64(values, nlimbs):
    buf = b"".join(int(v).to_bytes(8 * nlimbs, "little") for v in values)
    return np.frombuffer(buf, dtype="<u8").reshape(len(values), nlimbs).copy()


def _ints(arr):
    arr = np.ascontiguousarray(arr, dtype="<u8")
    nb = arr.shape[1] * 8
    raw = arr.tobytes()
    return [int.from_bytes(raw[i * nb:(i + 1) * nb], "little") for i in range(arr.shape[0])]


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class CKey:
    """paillier_z key in the C restatement (ciphertexts: uint64 (count, k/32))."""

    def __init__(self, key_bits, pk, sk=None, window=10):
        self.lib = load()
        self.key_bits = key_bits
        self.s = key_bits // 32
        h = self.s // 4
        self.pk, self.sk = pk, sk
        n = _u64([pk.n], self.s // 2)
        hs = _u64([pk.h_s], self.s)
        args = [None] * 7
        if sk is not None:
            R = 1 << (64 * h)
            args = [_u64([v], h) for v in (sk.p, sk.q, sk.hp, sk.hq, sk.pinv_q, pow(sk.p, -1, R), pow(sk.q, -1, R))]
        self._keep = [n, hs] + args
        self.h = self.lib.pz_key_create(key_bits, _p(n), _p(hs), *[_p(a) for a in args], window)
        if not self.h:
            raise MemoryError("pz_key_create failed")
        self.r_limbs = key_bits // 128

    def __del__(self):
        try:
            self.lib.pz_key_free(self.h)
        except Exception:
            pass

    def r_array(self, rs):
        return _u64(rs, self.r_limbs)

    def cts(self, mont_values):
        return _u64(mont_values, self.s)

    def ints(self, arr):
        return _ints(arr)

    def encrypt(self, m, r, threads=1):
        m = np.ascontiguousarray(m, dtype=np.int64)
        out = np.empty((m.size, self.s), dtype=np.uint64)
        rc = self.lib.pz_encrypt(self.h, _p(m), _p(r), _p(out), m.size, threads)
        assert rc == 0
        return out

    def decrypt(self, ct, threads=1):
        out = np.empty(ct.shape[0], dtype=np.int64)
        ovf = np.empty(ct.shape[0], dtype=np.uint8)
        rc = self.lib.pz_decrypt(self.h, _p(ct), _p(out), _p(ovf), ct.shape[0], threads)
        assert rc == 0
        return out, ovf

    def add(self, a, b, threads=1):
        out = np.empty_like(a)
        assert self.lib.pz_add(self.h, _p(a), _p(b), _p(out), a.shape[0], threads) == 0
        return out

    def mul(self, a, k, threads=1):
        k = np.ascontiguousarray(k, dtype=np.int64)
        out = np.empty_like(a)
        assert self.lib.pz_mul(self.h, _p(a), _p(k), _p(out), a.shape[0], threads) == 0
        return out

    def sum(self, a):
        out = np.empty((1, self.s), dtype=np.uint64)
        assert self.lib.pz_sum(self.h, _p(a), a.shape[0], _p(out)) == 0
        return out

    def sum_mt(self, a, threads=1):
        out = np.empty((1, self.s), dtype=np.uint64)
        assert self.lib.pz_sum_mt(self.h, _p(np.ascontiguousarray(a)), a.shape[0], _p(out), threads) == 0
        return out

    def bucket_sum(self, x, order_map, buckets, threads=1):
        """x (rows, s) ciphertexts, order_map (rows, F) uint8 -> (F * buckets, s)."""
        x = np.ascontiguousarray(x)
        om = np.ascontiguousarray(order_map, dtype=np.uint8)
        F = om.shape[1]
        out = np.empty((F * buckets, self.s), dtype=np.uint64)
        assert self.lib.pz_bucket_sum(self.h, _p(x), x.shape[0], _p(om), F, buckets, _p(out), threads) == 0
        return out

    def matmul(self, x, y, threads=1):
        """x (M, K, s) ciphertexts, y (K, N) int64 -> (M, N, s)."""
        x = np.ascontiguousarray(x)
        y = np.ascontiguousarray(y, dtype=np.int64)
        M, K, N = x.shape[0], x.shape[1], y.shape[1]
        out = np.empty((M, N, self.s), dtype=np.uint64)
        assert self.lib.pz_matmul(self.h, _p(x), M, K, _p(y), N, _p(out), threads) == 0
        return out

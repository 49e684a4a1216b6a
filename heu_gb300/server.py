"""Continuous-batching request server (hg_server_* of the C-ABI).

Requests carry host buffers (NumPy arrays) or handles of ciphertext vectors
kept resident on the device; results are bit-identical to the same request
run alone.  ``submit`` returns a ticket, ``wait`` blocks until the request is
done and returns its latency in seconds.
"""

import ctypes

import numpy as np

from heu_gb300 import capi

ENCRYPT, DECRYPT, ADD, MUL, SUM = (capi.HG_OP_ENCRYPT, capi.HG_OP_DECRYPT, capi.HG_OP_ADD, capi.HG_OP_MUL,
                                   capi.HG_OP_SUM)


def _p(a):
    return a.ctypes.data if a is not None else None


class Server:
    SHORTEST, FIFO = 0, 1

    def __init__(self, ctx, budget_bytes=0, slots=0, max_batch_elems=0, variant=0, batch_us=0.0, slice_us=0.0,
                 policy=0, express_us=0.0, express_share=0.0, express_len=0):
        self.ctx = ctx
        self.lib = ctx.lib
        cfg = capi.ServerConfig(budget_bytes, slots, max_batch_elems, variant, batch_us, slice_us, policy,
                                express_us, express_share, express_len)
        h = ctypes.c_void_p()
        capi.check(self.lib.hg_server_create(ctx.handle, ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h
        self._keep = {}

    def store(self, key, ct):
        """Copy ciphertexts (count, S) to a resident device vector; returns its handle."""
        ct = np.ascontiguousarray(ct, dtype=np.uint32).reshape(-1, key.ct_limbs)
        hd = ctypes.c_uint64()
        capi.check(self.lib.hg_server_store(self.handle, key.id, ctypes.c_void_p(ct.ctypes.data), ct.shape[0],
                                            ctypes.byref(hd)))
        return hd.value

    def release(self, handle):
        capi.check(self.lib.hg_server_release(self.handle, handle))

    def submit(self, key, op, count, in0=None, in1=None, h0=0, h1=0, out=None, aux=None):
        """Queue a request; all arrays must stay alive until wait() returns."""
        req = capi.Request(key.id, op, count, _p(in0), _p(in1), h0, h1, _p(out), _p(aux))
        t = ctypes.c_uint64()
        capi.check(self.lib.hg_server_submit(self.handle, ctypes.byref(req), ctypes.byref(t)))
        self._keep[t.value] = (in0, in1, out, aux)
        return t.value

    def wait(self, ticket):
        lat = ctypes.c_double()
        rc = self.lib.hg_server_wait(self.handle, ticket, ctypes.byref(lat))
        self._keep.pop(ticket, None)
        capi.check(rc)
        return lat.value

    def stats(self):
        c, b = ctypes.c_uint64(), ctypes.c_uint64()
        i, p = ctypes.c_size_t(), ctypes.c_size_t()
        capi.check(self.lib.hg_server_stats(self.handle, ctypes.byref(c), ctypes.byref(b), ctypes.byref(i),
                                            ctypes.byref(p)))
        return {"completed": c.value, "batches": b.value, "inflight_bytes": i.value, "pending": p.value}

    def trace_start(self):
        """Start a per-batch trace (clears the previous one)."""
        capi.check(self.lib.hg_probe_server_trace(self.handle, 1, None, 0, None))

    def trace_stop(self):
        """Stop the trace; returns one row per retired batch (a (batches, 12)
        float64 array): slot, class (0 regular, 1 express, 2 slow express),
        slices, elements, op mask (bit per op), host times formed / launched /
        retired and the GPU start time (seconds since trace_start), and the
        milliseconds the slot's stream spent on staged copies, kernels and
        copies back."""
        n = ctypes.c_size_t()
        capi.check(self.lib.hg_probe_server_trace(self.handle, 0, None, 0, ctypes.byref(n)))
        recs = np.zeros((n.value, 12), dtype=np.float64)
        if n.value:
            capi.check(self.lib.hg_probe_server_trace(self.handle, 0, ctypes.c_void_p(recs.ctypes.data), n.value,
                                                      ctypes.byref(n)))
        return recs

    def close(self):
        if self.handle:
            self.lib.hg_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

"""Persistent multi-key batches (hg_batch_* of the C-ABI).

A batch collects jobs on device buffers — any loaded key (1024/2048/3072
bits), any of encrypt / decrypt / add / scalar mul — and runs them in one
persistent kernel launch, optionally captured once into a CUDA graph and
replayed.  Device buffers are passed as raw device addresses (int) or as
objects with ``data_ptr()`` (e.g. torch tensors).
"""

import ctypes

from heu_gb300 import capi

ENCRYPT, DECRYPT, ADD, MUL = capi.HG_OP_ENCRYPT, capi.HG_OP_DECRYPT, capi.HG_OP_ADD, capi.HG_OP_MUL
PER_KEY = capi.HG_BATCH_PER_KEY


def _addr(x):
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return ctypes.c_void_p(x.data_ptr())
    return ctypes.c_void_p(int(x))


def _stream(s):
    if s is None:
        return None
    if hasattr(s, "cuda_stream"):
        return ctypes.c_void_p(s.cuda_stream)
    return ctypes.c_void_p(int(s))


class Batch:
    def __init__(self, ctx):
        self.ctx = ctx
        self.lib = ctx.lib
        h = ctypes.c_void_p()
        capi.check(self.lib.hg_batch_create(ctx.handle, ctypes.byref(h)))
        self.handle = h
        self.jobs = []

    def add(self, key, op, count, in0, in1=None, out=None, aux=None, nonneg=False):
        """Append a job; see include/heu_gb300.h for the operand meaning."""
        flags = capi.HG_JOB_NONNEG if nonneg else 0
        capi.check(self.lib.hg_batch_add(self.handle, key.id, op, count, _addr(in0), _addr(in1), _addr(out),
                                         _addr(aux), flags))
        self.jobs.append((key, op, count))

    def clear(self):
        capi.check(self.lib.hg_batch_clear(self.handle))
        self.jobs = []

    def set_variant(self, variant):
        """0 or 1: every job in that layout variant set; PER_KEY: each job in
        its key's tuned layout, one persistent launch per set in use."""
        capi.check(self.lib.hg_batch_set_variant(self.handle, variant))

    def run(self, stream=None, graph=False):
        capi.check(self.lib.hg_batch_run(self.handle, _stream(stream), 1 if graph else 0))

    def wait(self, stream=None):
        capi.check(self.lib.hg_batch_wait(self.handle, _stream(stream)))

    def close(self):
        if self.handle:
            self.lib.hg_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

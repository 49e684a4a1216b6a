"""Byte parity of Encrypt at the fixed-base table windows the throughput
benchmark uses: window 20 (52 table positions of 2^20 - 1 entries, 27.9 GB at
2048 bits, a 4-bit top digit) and window 16 (64 positions, 2.1 GB).

The r stream is chosen so that every table position sees its extreme digits:
all-ones digits, zero digits, a single set digit per position, alternating
digits and the short top digit; the rest are uniform 1024-bit values.  Every
ciphertext is compared in Montgomery form with the C restatement of
paillier_z (encryptor.cc:26-56 with HEU's window-10 table) and a sample in
Z-form with the Python oracle.  A decrypt round trip cannot catch a wrong
h_s^r (any r decrypts correctly), so this is the only check of the table
indexing at these windows.
"""

import os

import numpy as np
import pytest

import heu_gb300 as hg
from oracle import cref
from oracle import paillier_z as pz
from oracle.prg import Prg

from tests.conftest import oracle_key

pytestmark = pytest.mark.gpu

RBITS = 1024


def edge_randomness(w):
    """r values that drive every w-bit digit position to its extremes."""
    npos = -(-RBITS // w)
    full = (1 << RBITS) - 1
    dmax = (1 << w) - 1
    rs = [0, 1, 2, full, full - 1, 1 << (RBITS - 1)]
    for pos in range(npos):
        rs.append((dmax << (pos * w)) & full)       # one all-ones digit
        rs.append(1 << (pos * w))                   # one digit equal to 1
        rs.append(full ^ ((dmax << (pos * w)) & full))  # every digit full but this one
    rs.append(sum(dmax << (p * w) for p in range(0, npos, 2)) & full)  # alternating digits
    rs.append(sum(dmax << (p * w) for p in range(1, npos, 2)) & full)
    top = (npos - 1) * w
    rs += [((1 << (RBITS - top)) - 1) << top, 1 << top, full >> 1]  # the short top digit
    return rs


@pytest.mark.parametrize("window", [20, 16])
def test_encrypt_bytes_at_bench_window(gpu_ctx, window):
    pk, sk = oracle_key(2048, 0)
    key = gpu_ctx.load_key(2048, pk.n, pk.h_s, sk.p, sk.q, table_window=window)
    try:
        prg = Prg(70 + window)
        rs = edge_randomness(window)
        n = 4096
        rs += [prg.below(1 << RBITS) for _ in range(n - len(rs))]
        ms = [0, 1, -1, 2 ** 40 - 1, -(2 ** 40)] + [prg.int64_uniform(-(2 ** 40), 2 ** 40) for _ in range(n - 5)]
        m = np.array(ms, dtype=np.int64)
        ct = key.encrypt(m, hg.ints_to_limbs(rs, key.r_limbs))
        ck = cref.CKey(2048, pk, sk, window=10)
        want = ck.encrypt(m, ck.r_array(rs), threads=os.cpu_count() or 1)
        got = np.ascontiguousarray(ct, dtype=np.uint32)
        bad = np.nonzero((got != want.view(np.uint32).reshape(got.shape)).any(axis=1))[0]
        assert bad.size == 0, f"window {window}: {bad.size} Montgomery-form mismatches, first at {bad[:4]}"
        # Z-form against the definitional oracle on the edge cases and a sample
        idx = list(range(len(edge_randomness(window)))) + list(range(n - 64, n))
        z = hg.limbs_to_ints(key.from_mont(got[idx]))
        assert z == [pz.encrypt(pk, ms[i], rs[i]) for i in idx], f"window {window}: Z-form mismatch"
        # full-range plaintexts at the bound +-n/2 (encryptor.cc:38-40)
        half = pk.n // 2
        big = [half, -half, half - 1, -(half - 1)]
        rb = rs[:4]
        cb = key.encrypt_bn(big, hg.ints_to_limbs(rb, key.r_limbs))
        assert hg.limbs_to_ints(key.from_mont(cb)) == [pz.encrypt(pk, v, r) for v, r in zip(big, rb)]
    finally:
        key.free()

"""The allocation-free Sum (hg_dev_sum_noalloc), for callers that cannot call
cudaMalloc because their device memory belongs to another allocator or is
reserved up front.  It must give exactly what hg_dev_sum gives, call after
call, although its partial products live in one fixed device array shared by
every call.  This file is named so pytest collects it last."""

import ctypes

import numpy as np
import pytest

import heu_gb300 as hg
from heu_gb300 import capi

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _encrypt_on_device(torch, key, n, seed):
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    m = torch.randint(-(2 ** 40), 2 ** 40, (n,), dtype=torch.int64, device=dev, generator=g)
    r = torch.randint(-(2 ** 31), 2 ** 31, (n, key.r_limbs), dtype=torch.int32, device=dev, generator=g)
    ct = torch.empty((n, key.ct_limbs), dtype=torch.int32, device=dev)
    capi.check(key.lib.hg_dev_encrypt(key.ctx.handle, key.id, _ptr(m), _ptr(r), _ptr(ct), n, None))
    torch.cuda.synchronize()
    return m, ct


def test_noalloc_sum_matches_hg_dev_sum_twice(gpu_key):
    torch = pytest.importorskip("torch")
    key, pk, sk = gpu_key(2048, 0)
    lib, h = key.lib, key.ctx.handle
    for n, seed in ((300_000, 5), (4097, 6)):
        m, ct = _encrypt_on_device(torch, key, n, seed)
        want = torch.zeros((1, key.ct_limbs), dtype=torch.int32, device="cuda")
        got = torch.full((1, key.ct_limbs), -1, dtype=torch.int32, device="cuda")
        capi.check(lib.hg_dev_sum(h, key.id, _ptr(ct), n, _ptr(want), None))
        torch.cuda.synchronize()
        capi.check(lib.hg_dev_check(h))
        capi.check(lib.hg_dev_sum_noalloc(h, key.id, _ptr(ct), n, _ptr(got), None))
        torch.cuda.synchronize()
        assert torch.equal(got, want), f"noalloc sum differs from hg_dev_sum at n={n}"
        dm, ovf = key.decrypt(got.cpu().numpy().view(np.uint32))
        assert int(dm[0]) == int(m.sum().item()) and ovf[0] == 0


def test_noalloc_sum_rejects_counts_beyond_its_scratch(gpu_key):
    torch = pytest.importorskip("torch")
    key, pk, sk = gpu_key(2048, 0)
    buf = torch.zeros((2, key.ct_limbs), dtype=torch.int32, device="cuda")
    too_many = 128 * (((16 << 20) - 256) // (8 * key.ct_limbs)) + 1
    rc = key.lib.hg_dev_sum_noalloc(key.ctx.handle, key.id, _ptr(buf), too_many, _ptr(buf), None)
    assert rc == capi.HG_ERR_INVALID
    assert b"fixed scratch" in key.lib.hg_last_error()
    # a single ciphertext and a range error still behave like hg_dev_sum
    bad = torch.from_numpy(hg.ints_to_limbs([pk.n2, 3], key.ct_limbs).view(np.int32)).cuda()
    out = torch.zeros((1, key.ct_limbs), dtype=torch.int32, device="cuda")
    rc = key.lib.hg_dev_sum_noalloc(key.ctx.handle, key.id, _ptr(bad), 2, _ptr(out), None)
    assert rc == capi.HG_ERR_CT_RANGE


def test_noalloc_sum_checks_every_input(gpu_key):
    """One value >= n^2 anywhere in the input, not only at the start of a
    reduction chunk, is rejected; a valid call right after still sums."""
    torch = pytest.importorskip("torch")
    key, pk, sk = gpu_key(2048, 0)
    lib, h = key.lib, key.ctx.handle
    m, ct = _encrypt_on_device(torch, key, 300_000, 7)
    n2 = torch.from_numpy(hg.ints_to_limbs([pk.n2 + 3], key.ct_limbs).view(np.int32)).cuda()
    out = torch.zeros((1, key.ct_limbs), dtype=torch.int32, device="cuda")
    for n, bad_at in ((2, 1), (64, 63), (300_000, 1), (300_000, 12_345)):
        x = ct[:n].clone()
        x[bad_at] = n2[0]
        torch.cuda.synchronize()  # the engine's stream does not wait for torch's
        rc = lib.hg_dev_sum_noalloc(h, key.id, _ptr(x), n, _ptr(out), None)
        assert rc == capi.HG_ERR_CT_RANGE, (n, bad_at)
    want = torch.zeros_like(out)
    capi.check(lib.hg_dev_sum(h, key.id, _ptr(ct), 300_000, _ptr(want), None))
    torch.cuda.synchronize()
    capi.check(lib.hg_dev_check(h))
    capi.check(lib.hg_dev_sum_noalloc(h, key.id, _ptr(ct), 300_000, _ptr(out), None))
    assert torch.equal(out, want)

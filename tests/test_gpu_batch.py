"""Persistent multi-key batches and the autotuner: a batch of uneven jobs
across 1024/2048/3072-bit keys gives exactly the per-call results, eagerly
and replayed from a captured CUDA graph, under both layout variants; every
layout variant is bit-exact against the oracle."""

import ctypes

import numpy as np
import pytest

import heu_gb300 as hg
from heu_gb300 import autotune, capi
from heu_gb300.batch import ADD, DECRYPT, ENCRYPT, MUL
from oracle import paillier_z as pz

pytestmark = pytest.mark.gpu

KEYS = [(1024, 1), (2048, 0), (3072, 2)]


def P(t):
    return ctypes.c_void_p(t.data_ptr())


def _inputs(torch, key, n, seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    m = torch.randint(-(2 ** 62), 2 ** 62, (n,), dtype=torch.int64, device="cuda", generator=g)
    r = torch.randint(-(2 ** 31), 2 ** 31, (n, key.r_limbs), dtype=torch.int32, device="cuda", generator=g)
    k = torch.randint(-(2 ** 63), 2 ** 63 - 1, (n,), dtype=torch.int64, device="cuda", generator=g)
    return m, r, k


def _ct(torch, key, n):
    return torch.empty((n, key.ct_limbs), dtype=torch.int32, device="cuda")


def _build_jobs(torch, keys, sizes):
    """Per key: encrypt, mul (signed k), add, decrypt jobs with their per-call expected outputs."""
    jobs = []
    for ki, (key, n) in enumerate(zip(keys, sizes)):
        lib, h = key.lib, key.ctx.handle
        m, r, k = _inputs(torch, key, n, 100 + ki)
        base = _ct(torch, key, n)
        capi.check(lib.hg_dev_encrypt(h, key.id, P(m), P(r), P(base), n, None))
        want_mul = _ct(torch, key, n)
        capi.check(lib.hg_dev_mul(h, key.id, P(base), P(k), P(want_mul), n, None))
        want_add = _ct(torch, key, n)
        capi.check(lib.hg_dev_add(h, key.id, P(base), P(want_mul), P(want_add), n, None))
        torch.cuda.synchronize()
        jobs.append(dict(key=key, n=n, m=m, r=r, k=k, base=base, want_mul=want_mul, want_add=want_add,
                         out_enc=_ct(torch, key, n), out_mul=_ct(torch, key, n), out_add=_ct(torch, key, n),
                         out_dec=torch.empty((n,), dtype=torch.int64, device="cuda"),
                         ovf=torch.empty((n,), dtype=torch.uint8, device="cuda")))
    return jobs


def _fill(batch, jobs):
    for j in jobs:
        key, n = j["key"], j["n"]
        batch.add(key, ENCRYPT, n, j["m"], j["r"], j["out_enc"])
        batch.add(key, MUL, n, j["base"], j["k"], j["out_mul"])
        batch.add(key, ADD, n, j["base"], j["want_mul"], j["out_add"])
        batch.add(key, DECRYPT, n, j["base"], None, j["out_dec"], j["ovf"])


def _check(torch, jobs):
    for j in jobs:
        assert torch.equal(j["out_enc"], j["base"]), f"encrypt k{j['key'].key_bits}"
        assert torch.equal(j["out_mul"], j["want_mul"]), f"mul k{j['key'].key_bits}"
        assert torch.equal(j["out_add"], j["want_add"]), f"add k{j['key'].key_bits}"
        assert torch.equal(j["out_dec"], j["m"]), f"decrypt k{j['key'].key_bits}"
        assert int(j["ovf"].sum().item()) == 0


def _zero(jobs):
    for j in jobs:
        for name in ("out_enc", "out_mul", "out_add", "out_dec"):
            j[name].zero_()


@pytest.mark.parametrize("variant", [0, 1])
def test_batch_matches_per_call_eager_and_graph(gpu_ctx, gpu_key, variant):
    torch = pytest.importorskip("torch")
    keys = [gpu_key(b, s)[0] for b, s in KEYS]
    jobs = _build_jobs(torch, keys, [517, 64, 33])
    batch = hg.Batch(gpu_ctx)
    batch.set_variant(variant)
    _fill(batch, jobs)
    batch.run(graph=False)
    batch.wait()
    _check(torch, jobs)
    for _ in range(2):  # capture, then replay
        _zero(jobs)
        batch.run(graph=True)
        batch.wait()
        _check(torch, jobs)
    batch.close()


def test_batch_per_key_variants(gpu_ctx, gpu_key):
    """HG_BATCH_PER_KEY: each job in its key's tuned layout (decryptions in
    the key's dec_variant), one launch per variant set; results unchanged."""
    torch = pytest.importorskip("torch")
    keys = [gpu_key(b, s)[0] for b, s in KEYS]
    saved = [autotune.get_config(k) for k in keys]
    try:
        # both variant sets in use, crossed between the n^2 and p^2 layouts
        for k, (v, dv) in zip(keys, [(1, 0), (0, 1), (1, 1)]):
            autotune.set_config(k, dict(autotune.get_config(k), variant=v, dec_variant=dv))
        jobs = _build_jobs(torch, keys, [300, 129, 70])
        batch = hg.Batch(gpu_ctx)
        batch.set_variant(hg.batch.PER_KEY)
        _fill(batch, jobs)
        batch.run(graph=False)
        batch.wait()
        _check(torch, jobs)
        _zero(jobs)
        batch.run(graph=True)
        batch.wait()
        _check(torch, jobs)
        batch.close()
    finally:
        for k, c in zip(keys, saved):
            autotune.set_config(k, c)


def test_batch_reports_range_errors(gpu_ctx, gpu_key):
    torch = pytest.importorskip("torch")
    key, pk, sk = gpu_key(1024, 1)
    bad = torch.from_numpy(hg.ints_to_limbs([pk.n2, 1], key.ct_limbs).view(np.int32)).cuda()
    out = torch.empty((2,), dtype=torch.int64, device="cuda")
    ovf = torch.empty((2,), dtype=torch.uint8, device="cuda")
    batch = hg.Batch(gpu_ctx)
    batch.add(key, DECRYPT, 2, bad, None, out, ovf)
    batch.run()
    with pytest.raises(hg.HgError) as ei:
        batch.wait()
    assert ei.value.code == capi.HG_ERR_CT_RANGE
    batch.close()


@pytest.mark.parametrize("bits,seed", KEYS, ids=lambda v: str(v))
def test_every_layout_variant_matches_oracle(gpu_ctx, bits, seed):
    from tests.conftest import oracle_key

    pk, sk = oracle_key(bits, seed)
    key = gpu_ctx.load_key(bits, pk.n, pk.h_s, sk.p, sk.q, table_window=8)
    ms = [0, 1, -1, 2 ** 62, -(2 ** 40), 12345]
    ks = [0, -1, 2, 2 ** 63 - 1, -(2 ** 63), 77]
    rs = pz.r_stream(70, len(ms), pk.key_size // 2)
    zs = [pz.encrypt(pk, m, r) for m, r in zip(ms, rs)]
    for v in (0, 1):
        for wm, wd in ((3, 4), (5, 6)):
            autotune.set_config(key, {"variant": v, "dec_variant": v, "mul_window": wm, "dec_window": wd})
            ct = key.encrypt(np.array(ms, dtype=np.int64), hg.ints_to_limbs(rs, key.r_limbs))
            assert hg.limbs_to_ints(key.from_mont(ct)) == zs, f"encrypt v{v}"
            mu = key.mul(ct, np.array(ks, dtype=np.int64))
            assert hg.limbs_to_ints(key.from_mont(mu)) == [pz.mul(pk, z, k) for z, k in zip(zs, ks)], f"mul v{v}"
            d, ovf = key.decrypt(ct)
            assert d.tolist() == ms and ovf.sum() == 0, f"decrypt v{v} wd{wd}"
    key.free()


def test_autotune_applies_a_valid_configuration(gpu_ctx, tmp_path):
    from tests.conftest import oracle_key

    pk, sk = oracle_key(1024, 1)
    key = gpu_ctx.load_key(1024, pk.n, pk.h_s, sk.p, sk.q, table_window=8)
    cfg, rates = autotune.tune(key, calib=4096)
    assert cfg["variant"] in (0, 1) and cfg["dec_variant"] in (0, 1)
    assert 3 <= cfg["mul_window"] <= 5 and 4 <= cfg["dec_window"] <= 6
    assert autotune.get_config(key) == cfg
    assert rates["encrypt"] > 0 and rates["mul"] > 0 and rates["decrypt"] > 0
    path = str(tmp_path / "tuning.json")
    autotune.save(cfg, 1024, path=path, rates=rates)
    assert autotune.load(1024, path=path) == cfg
    ms = [5, -6]
    rs = pz.r_stream(71, 2, pk.key_size // 2)
    ct = key.encrypt(np.array(ms, dtype=np.int64), hg.ints_to_limbs(rs, key.r_limbs))
    assert hg.limbs_to_ints(key.from_mont(ct)) == [pz.encrypt(pk, m, r) for m, r in zip(ms, rs)]
    key.free()

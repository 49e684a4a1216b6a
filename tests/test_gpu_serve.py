"""The continuous-batching server: requests of mixed keys, ops and lengths,
submitted concurrently from several threads, each give exactly the result
of the same request run alone through the per-call C-ABI."""

import threading

import numpy as np
import pytest

import heu_gb300 as hg
from heu_gb300 import capi
from heu_gb300.server import ADD, DECRYPT, ENCRYPT, MUL, SUM
from oracle import paillier_z as pz

pytestmark = pytest.mark.gpu


def _alone(key, op, x0, x1):
    if op == ENCRYPT:
        return key.encrypt(x0, x1)
    if op == DECRYPT:
        return key.decrypt(x0)[0]
    if op == ADD:
        return key.add(x0, x1)
    if op == MUL:
        return key.mul(x0, x1)
    return key.sum(x0)


@pytest.mark.parametrize("policy,express_len", [(hg.Server.SHORTEST, 0), (hg.Server.FIFO, 0),
                                                 (hg.Server.SHORTEST, 512)],
                         ids=["shortest", "fifo", "latency-class"])
def test_served_results_equal_alone(gpu_ctx, gpu_key, policy, express_len):
    """With express_len the requests of at most 512 elements run in the three
    express slots (one for short decryptions, two for the other short
    requests) in the latency layout; results stay identical."""
    keys = [gpu_key(2048, 0)[0], gpu_key(3072, 2)[0], gpu_key(1024, 1)[0]]
    rng = np.random.default_rng(17)
    server = hg.Server(gpu_ctx, budget_bytes=2 << 30, slots=5 if express_len else 3, max_batch_elems=1 << 14,
                       policy=policy, express_len=express_len)
    # one resident vector per key
    vec_len = 3000
    residents, res_host = [], []
    for key in keys:
        m = rng.integers(-(2 ** 40), 2 ** 40, size=vec_len)
        r = rng.integers(0, 2 ** 32, size=(vec_len, key.r_limbs), dtype=np.uint64).astype(np.uint32)
        ct = key.encrypt(m, r)
        res_host.append(ct)
        residents.append(server.store(key, ct))
    reqs = []
    for i in range(60):
        ki = int(rng.integers(3))
        key = keys[ki]
        n = int(np.floor(np.exp(rng.uniform(0, np.log(vec_len)))))
        op = [ENCRYPT, ADD, MUL, SUM, DECRYPT][int(rng.choice(5, p=[0.3, 0.2, 0.25, 0.15, 0.1]))]
        use_handle = bool(rng.integers(2)) and op != ENCRYPT
        if op == ENCRYPT:
            x0 = rng.integers(-(2 ** 63), 2 ** 63 - 1, size=n)
            x1 = rng.integers(0, 2 ** 32, size=(n, key.r_limbs), dtype=np.uint64).astype(np.uint32)
        else:
            x0 = res_host[ki][:n].copy()
            x1 = None
            if op == ADD:
                x1 = np.roll(x0, 1, axis=0) if not use_handle else res_host[ki][:n].copy()
            if op == MUL:
                x1 = rng.integers(-(2 ** 63), 2 ** 63 - 1, size=n)
        out = (np.empty(n, np.int64) if op == DECRYPT else
               np.empty((1 if op == SUM else n, key.ct_limbs), np.uint32))
        reqs.append(dict(key=key, ki=ki, op=op, n=n, x0=x0, x1=x1, out=out, h=use_handle))
    tickets = [None] * len(reqs)

    def submit(idx):
        for i in idx:
            q = reqs[i]
            h0 = residents[q["ki"]] if q["h"] else 0
            h1 = residents[q["ki"]] if (q["h"] and q["op"] == ADD) else 0
            in0 = None if h0 else q["x0"]
            in1 = None if h1 else q["x1"]
            tickets[i] = server.submit(q["key"], q["op"], q["n"], in0=in0, in1=in1, h0=h0, h1=h1, out=q["out"])

    b0 = server.stats()["batches"]
    server.trace_start()
    ths = [threading.Thread(target=submit, args=(list(range(t, len(reqs), 4)),)) for t in range(4)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    lats = [server.wait(t) for t in tickets]
    assert all(v >= 0 for v in lats)
    st = server.stats()
    assert st["completed"] == len(reqs) and st["pending"] == 0
    # one trace record per batch, in the classes this configuration has
    tr = server.trace_stop()
    assert len(tr) == st["batches"] - b0
    assert set(np.unique(tr[:, 1])) <= ({0, 1, 2} if express_len else {0})
    if express_len:
        assert (tr[tr[:, 1] > 0, 3] <= express_len).all()
        assert (tr[tr[:, 1] == 2, 4] == 2).all()  # the slow express slot runs decryptions only
        assert set(np.unique(tr[tr[:, 1] == 1, 0])) <= {0, 2}  # the two express slots of the rest
        assert set(np.unique(tr[tr[:, 1] == 0, 0])) <= {3, 4}
    assert (tr[:, 3] >= 1).all() and (tr[:, 4] > 0).all()
    assert (tr[:, 5] <= tr[:, 6]).all() and (tr[:, 6] <= tr[:, 7]).all()
    assert (tr[:, 9:12] >= 0).all()
    for q in reqs:
        x0 = q["x0"]
        x1 = q["x1"]
        want = _alone(q["key"], q["op"], x0, x1)
        assert np.array_equal(np.asarray(want).reshape(q["out"].shape), q["out"]), \
            f"op {q['op']} n {q['n']} k{q['key'].key_bits}"
    server.close()


@pytest.mark.parametrize("express_us", [2000.0, 0.0], ids=["express", "no-express"])
def test_long_requests_are_sliced_and_stay_exact(gpu_ctx, gpu_key, express_us):
    """Requests far longer than one slice (tiny slice budget) still give the
    per-call result, interleaved with short ones, with and without the
    express slot (which takes the 3-element request here)."""
    key, pk, sk = gpu_key(2048, 0)
    server = hg.Server(gpu_ctx, budget_bytes=1 << 30, slots=2, slice_us=50.0, batch_us=400.0,
                       express_us=express_us)
    rng = np.random.default_rng(23)
    n = 5000
    m = rng.integers(-(2 ** 40), 2 ** 40, size=n)
    r = rng.integers(0, 2 ** 32, size=(n, key.r_limbs), dtype=np.uint64).astype(np.uint32)
    k = rng.integers(-(2 ** 63), 2 ** 63 - 1, size=n)
    ct = np.empty((n, key.ct_limbs), np.uint32)
    t1 = server.submit(key, ENCRYPT, n, in0=m, in1=r, out=ct)
    small = np.empty((3, key.ct_limbs), np.uint32)
    t2 = server.submit(key, ENCRYPT, 3, in0=m[:3], in1=r[:3], out=small)
    server.wait(t2)
    server.wait(t1)
    assert np.array_equal(ct, key.encrypt(m, r))
    assert np.array_equal(small, ct[:3])
    mul = np.empty_like(ct)
    dec = np.empty(n, np.int64)
    ovf = np.empty(n, np.uint8)
    t3 = server.submit(key, MUL, n, in0=ct, in1=k, out=mul)
    t4 = server.submit(key, DECRYPT, n, in0=ct, out=dec, aux=ovf)
    server.wait(t3)
    server.wait(t4)
    assert np.array_equal(mul, key.mul(ct, k))
    assert np.array_equal(dec, m) and ovf.sum() == 0
    assert server.stats()["batches"] > 4
    server.close()


def test_server_rejects_bad_requests(gpu_ctx, gpu_key):
    key, pk, sk = gpu_key(1024, 1)
    server = hg.Server(gpu_ctx, budget_bytes=64 << 20, slots=2)
    with pytest.raises(hg.HgError) as ei:
        server.submit(key, DECRYPT, 4, h0=999, out=np.empty(4, np.int64))
    assert ei.value.code == capi.HG_ERR_INVALID
    big = np.zeros((1 << 20, key.ct_limbs), np.uint32)
    with pytest.raises(hg.HgError) as ei:  # a sum is never sliced: it must fit one slot
        server.submit(key, SUM, big.shape[0], in0=big, out=big[:1])
    assert ei.value.code == capi.HG_ERR_NOMEM
    bad = hg.ints_to_limbs([pk.n2, 1], key.ct_limbs)
    t = server.submit(key, DECRYPT, 2, in0=bad, out=np.empty(2, np.int64))
    with pytest.raises(hg.HgError) as ei:
        server.wait(t)
    assert ei.value.code == capi.HG_ERR_CT_RANGE
    # encryption through the server matches the oracle
    ms = np.array([3, -4, 5], dtype=np.int64)
    rs = pz.r_stream(90, 3, pk.key_size // 2)
    out = np.empty((3, key.ct_limbs), np.uint32)
    t = server.submit(key, ENCRYPT, 3, in0=ms, in1=hg.ints_to_limbs(rs, key.r_limbs), out=out)
    server.wait(t)
    assert hg.limbs_to_ints(key.from_mont(out)) == [pz.encrypt(pk, int(m), r) for m, r in zip(ms, rs)]
    server.close()

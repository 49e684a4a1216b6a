"""Sharded path over world-size-2 gloo ranks on CPU.

Each rank holds its shard of the ciphertexts; the reduction partials are
all-gathered and combined.  On this host the per-rank arithmetic is done by
the oracle standing in for the engine (a key-like object below), so what is
tested here is the host logic: shard bounds, partial exchange, combine order
and failure behaviour.  A rank that dies before the collective makes the
other rank's collective fail instead of hanging."""

import os
import socket
from datetime import timedelta

import numpy as np
import pytest

from heu_gb300.distributed import shard_bounds


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


class OracleKey:
    """Key-like object computing with the paillier_z oracle (Montgomery form
    in and out, as the engine's Key)."""

    def __init__(self, bits, seed):
        from oracle import paillier_z as pz

        self.pz = pz
        self.pk, self.sk = pz.keygen(bits, seed)
        self.ct_limbs = self.pk.S
        self.r_limbs = bits // 64

    def _z(self, arr):
        import heu_gb300 as hg

        return [self.pz.from_mont(self.pk, v) for v in hg.limbs_to_ints(arr.reshape(-1, self.ct_limbs))]

    def _m(self, zs):
        import heu_gb300 as hg

        return hg.ints_to_limbs([self.pz.to_mont(self.pk, z) for z in zs], self.ct_limbs)

    def encrypt(self, m, r):
        import heu_gb300 as hg

        rs = hg.limbs_to_ints(np.asarray(r, dtype=np.uint32).reshape(-1, self.r_limbs))
        return self._m([self.pz.encrypt(self.pk, int(v), rv) for v, rv in zip(np.asarray(m).reshape(-1), rs)])

    def sum(self, ct):
        return self._m([self.pz.sum_(self.pk, self._z(ct))])

    def add(self, a, b):
        return self._m([self.pz.add(self.pk, x, y) for x, y in zip(self._z(a), self._z(b))])

    def bucket_sum(self, x, om, buckets, cumsum=False):
        zs = self._z(x)
        rows = np.asarray(om).shape[0]
        cols = len(zs) // rows
        xm = [[zs[i * cols + c] for c in range(cols)] for i in range(rows)]
        res = self.pz.bucket_sum(self.pk, xm, np.asarray(om).tolist(), buckets, cumsum=cumsum)
        return self._m([v for row in res for v in row]).reshape(len(res), cols, self.ct_limbs)


def _data(key, n, feats, buckets):
    from oracle import paillier_z as pz

    rng = np.random.default_rng(3)
    m = rng.integers(-1000, 1000, size=n)
    rs = pz.r_stream(5, n, key.pk.key_size // 2)
    import heu_gb300 as hg

    ct = key.encrypt(m, hg.ints_to_limbs(rs, key.r_limbs))
    om = rng.integers(0, buckets, size=(n, feats)).astype(np.uint8)
    return m, ct, om


def _worker(rank, world, port, outdir, fail_rank):
    import torch.distributed as dist

    from heu_gb300.distributed import sharded_bucket_sum, sharded_sum

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world,
                            timeout=timedelta(seconds=15))
    try:
        if rank == fail_rank:
            raise SystemExit(3)  # this rank dies before the collective
        key = OracleKey(1024, 1)
        n, feats, buckets = 23, 2, 3
        m, ct, om = _data(key, n, feats, buckets)
        a, b = shard_bounds(n, rank, world)
        total = sharded_sum(key, ct[a:b])
        bs = sharded_bucket_sum(key, ct[a:b], om[a:b], buckets, cumsum=True)
        np.save(os.path.join(outdir, f"sum{rank}.npy"), total)
        np.save(os.path.join(outdir, f"bs{rank}.npy"), bs)
    except SystemExit:
        raise
    except Exception as e:  # record the failure mode for the parent
        with open(os.path.join(outdir, f"err{rank}.txt"), "w") as f:
            f.write(type(e).__name__ + ": " + str(e))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _run(world, fail_rank, tmp_path):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, str(tmp_path), fail_rank)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        if p.is_alive():
            p.kill()
            pytest.fail("a rank hung")
    return procs


def test_shard_bounds_cover_everything():
    for n in (0, 1, 5, 23, 1000):
        for world in (1, 2, 3, 8):
            spans = [shard_bounds(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def test_two_rank_sum_and_bucket_sum_equal_single_process(tmp_path):
    _run(2, -1, tmp_path)
    key = OracleKey(1024, 1)
    m, ct, om = _data(key, 23, 2, 3)
    want_sum = key.sum(ct)
    want_bs = key.bucket_sum(ct, om, 3, cumsum=True)
    for r in range(2):
        assert not (tmp_path / f"err{r}.txt").exists(), (tmp_path / f"err{r}.txt").read_text()
        assert np.array_equal(np.load(tmp_path / f"sum{r}.npy"), want_sum)
        assert np.array_equal(np.load(tmp_path / f"bs{r}.npy"), want_bs)
    from oracle import paillier_z as pz

    assert pz.decrypt(key.pk, key.sk, key._z(want_sum)[0]) == int(m.sum())


def test_a_dead_rank_fails_the_collective_instead_of_hanging(tmp_path):
    procs = _run(2, 1, tmp_path)
    assert procs[1].exitcode == 3
    err = tmp_path / "err0.txt"
    assert err.exists(), "rank 0 should have seen the collective fail"
    assert not (tmp_path / "sum0.npy").exists()

"""Sharding the Paillier path over ranks (one process per GPU).

Element-wise operations (encrypt, decrypt, add, scalar mul, negate) shard by
contiguous element ranges and need no exchange.  The heu.numpy reductions
have one exchange step: every rank reduces its shard to partial ciphertexts
(one for Sum, features x buckets for bucket-sum) and the partials are
combined with the scheme's addition (a modular product), which is
associative and commutative, so the combined result equals the
single-process one bit for bit.  MatMul shards the rows of the ciphertext
matrix and needs no exchange either.

Partials travel as uint32 limb tensors through torch.distributed
(all_gather); the combine then runs on the local engine.  The `key` objects
only need ``sum``, ``add`` and ``ct_limbs`` (heu_gb300.Key provides them).
"""

import numpy as np


def shard_bounds(n, rank, world):
    """Contiguous, balanced [start, end) of n elements for `rank`."""
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def _all_gather_limbs(arr, group=None):
    import torch
    import torch.distributed as dist

    t = torch.from_numpy(np.ascontiguousarray(arr).view(np.int32).copy())
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    world = dist.get_world_size(group)
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    return [p.cpu().numpy().view(np.uint32) for p in parts]


def _identity(key):
    """Montgomery identity (the encryption of 0 with r = 0): Sum's neutral element."""
    r = np.zeros((1, key.r_limbs), dtype=np.uint32)
    return key.encrypt(np.zeros(1, dtype=np.int64), r)


def sharded_sum(key, local_ct, group=None):
    """Sum (numpy/evaluator.cc:355-373) of a ciphertext vector sharded by rank."""
    local_ct = np.ascontiguousarray(local_ct, dtype=np.uint32).reshape(-1, key.ct_limbs)
    partial = key.sum(local_ct) if local_ct.shape[0] else _identity(key)
    parts = _all_gather_limbs(partial, group)
    return key.sum(np.concatenate(parts, axis=0))


def sharded_bucket_sum(key, local_x, local_order_map, bucket_num, cumsum=False, group=None):
    """FeatureWiseBucketSum with rows sharded by rank: per-rank bucket products,
    combined bucket by bucket across ranks (cumsum applied after the combine)."""
    partial = key.bucket_sum(local_x, local_order_map, bucket_num, cumsum=False)
    shape = partial.shape
    parts = _all_gather_limbs(partial.reshape(-1, key.ct_limbs), group)
    acc = parts[0]
    for p in parts[1:]:
        acc = key.add(acc, p)
    out = acc.reshape(shape)
    if cumsum:
        feats = shape[0] // bucket_num
        out = out.reshape(feats, bucket_num, -1, key.ct_limbs).copy()
        for b in range(1, bucket_num):
            out[:, b] = key.add(out[:, b - 1].reshape(-1, key.ct_limbs),
                                out[:, b].reshape(-1, key.ct_limbs)).reshape(out[:, b].shape)
        out = out.reshape(shape)
    return out


def sharded_matmul(key, local_rows, y, group=None, gather=False):
    """MatMul with the ciphertext matrix's rows sharded by rank; no exchange
    unless `gather` asks for the full result on every rank."""
    out = key.matmul(local_rows, y)
    if not gather:
        return out
    import torch
    import torch.distributed as dist

    # rows differ per rank: gather sizes first, then padded blocks
    world = dist.get_world_size(group)
    n = torch.tensor([out.shape[0]], dtype=torch.int64)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    mx = int(max(s.item() for s in sizes))
    pad = np.zeros((mx,) + out.shape[1:], dtype=np.uint32)
    pad[: out.shape[0]] = out
    parts = _all_gather_limbs(pad, group)
    return np.concatenate([p[: int(s.item())] for p, s in zip(parts, sizes)], axis=0)

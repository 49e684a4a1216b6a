"""Generate tests/golden/paillier_z_kat.json from the paillier_z oracle.

The reference cannot be built in this environment (Bazel + yacl), and its
own tests hold no ciphertext known-answer vectors, so these fixtures are the
oracle's outputs on seeded keys and seeded r streams; tests/test_oracle.py
pins the oracle itself against the reference tests' literal expectations.

Run:  python tests/golden/gen_golden.py
"""

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import paillier_z as pz  # noqa: E402

I64_MIN, I64_MAX = -(2 ** 63), 2 ** 63 - 1
MS = [0, 1, -1, -12345, 123, I64_MIN, I64_MAX, 2 ** 40 - 7]
KS = [0, 1, -1, 2, -2, 2 ** 15 - 1, -(2 ** 15), I64_MIN]
KS_MORE = [2 ** 31 - 1, -(2 ** 31), 0x5DEECE66D1234567, -0x2545F4914F6CDD1D]


def h(v):
    return format(v, "x")


def case(bits, seed, extras=False):
    pk, sk = pz.keygen(bits, seed)
    rs = pz.r_stream(seed + 100, len(MS), pk.key_size // 2)
    zs = [pz.encrypt(pk, m, r) for m, r in zip(MS, rs)]
    # full-range plaintexts +-(n/2 - 1) and the bounds +-n/2 (paillier_test.cc:190-205)
    big = [pk.n_half - 1, -(pk.n_half - 1), pk.n_half, -pk.n_half]
    rb = pz.r_stream(seed + 200, len(big), pk.key_size // 2)
    zb = [pz.encrypt(pk, m, r) for m, r in zip(big, rb)]
    out = {
        "key_bits": bits, "seed": seed,
        "n": h(pk.n), "p": h(sk.p), "q": h(sk.q), "h_s": h(pk.h_s),
        "m": [str(m) for m in MS], "r": [h(r) for r in rs],
        "ct_z": [h(z) for z in zs], "ct_mont": [h(pz.to_mont(pk, z)) for z in zs],
        "add_next": [h(pz.add(pk, zs[i], zs[(i + 1) % len(zs)])) for i in range(len(zs))],
        "sub_next": [h(pz.sub(pk, zs[i], zs[(i + 1) % len(zs)])) for i in range(len(zs))],
        "negate": [h(pz.negate(pk, z)) for z in zs],
        "k": [str(k) for k in KS],
        "mul": [h(pz.mul(pk, z, k)) for z, k in zip(zs, KS)],
        "k_more": [str(k) for k in KS_MORE],
        "mul_more": [h(pz.mul(pk, zs[i], k)) for i, k in enumerate(KS_MORE)],
        "sum": h(pz.sum_(pk, zs)),
        "add_plain": [h(pz.add_plain(pk, z, m)) for z, m in zip(zs, MS)],
        "m_big": [str(m) for m in big], "r_big": [h(r) for r in rb], "ct_big_z": [h(z) for z in zb],
    }
    if extras:
        # numpy_test.cc:111-120: Sum of the encryptions of 0..899 (decrypts to 404550)
        r900 = pz.r_stream(seed + 300, 900, pk.key_size // 2)
        z900 = [pz.encrypt(pk, m, r) for m, r in zip(range(900), r900)]
        out["sum_0_899"] = {"r_seed": seed + 300, "ct_z": h(pz.sum_(pk, z900))}
        # bucket-sum: 12 rows x 2 columns, 2 features, 3 buckets (with an empty bucket), cumsum both ways
        vals = [[(i * 7919) % 2001 - 1000, (i * 104729) % 2001 - 1000] for i in range(12)]
        om = [[i % 3 if i % 5 else 0, (i * 2) % 2] for i in range(12)]
        rr = pz.r_stream(seed + 400, 24, pk.key_size // 2)
        xz = [[pz.encrypt(pk, vals[i][c], rr[2 * i + c]) for c in range(2)] for i in range(12)]
        out["bucket_sum"] = {
            "vals": vals, "order_map": om, "buckets": 3, "r_seed": seed + 400,
            "out_z": [[h(v) for v in row] for row in pz.bucket_sum(pk, xz, om, 3, cumsum=False)],
            "out_cumsum_z": [[h(v) for v in row] for row in pz.bucket_sum(pk, xz, om, 3, cumsum=True)],
        }
        # MatMul 3x4 ciphertexts @ 4x2 plaintexts (matmul_test.cc shapes are small like this)
        xm = [[(i * 31 + j * 17) % 201 - 100 for j in range(4)] for i in range(3)]
        ym = [[(i * 13 + j * 7) % 65 - 32 for j in range(2)] for i in range(4)]
        rm = pz.r_stream(seed + 500, 12, pk.key_size // 2)
        xmz = [[pz.encrypt(pk, xm[i][j], rm[4 * i + j]) for j in range(4)] for i in range(3)]
        out["matmul"] = {"x": xm, "y": ym, "r_seed": seed + 500,
                         "out_z": [[h(v) for v in row] for row in pz.matmul(pk, xmz, ym)]}
    return out


def main():
    data = {"generator": "tests/golden/gen_golden.py",
            "cases": [case(1024, 1, extras=True), case(2048, 0), case(3072, 2)]}
    path = os.path.join(HERE, "paillier_z_kat.json")
    with open(path, "w") as f:
        json.dump(data, f, indent=1)
    print(path)


if __name__ == "__main__":
    main()

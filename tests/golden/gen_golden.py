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


def h(v):
    return format(v, "x")


def case(bits, seed):
    pk, sk = pz.keygen(bits, seed)
    rs = pz.r_stream(seed + 100, len(MS), pk.key_size // 2)
    zs = [pz.encrypt(pk, m, r) for m, r in zip(MS, rs)]
    out = {
        "key_bits": bits, "seed": seed,
        "n": h(pk.n), "p": h(sk.p), "q": h(sk.q), "h_s": h(pk.h_s),
        "m": [str(m) for m in MS], "r": [h(r) for r in rs],
        "ct_z": [h(z) for z in zs], "ct_mont": [h(pz.to_mont(pk, z)) for z in zs],
        "add_next": [h(pz.add(pk, zs[i], zs[(i + 1) % len(zs)])) for i in range(len(zs))],
        "negate": [h(pz.negate(pk, z)) for z in zs],
        "k": [str(k) for k in KS],
        "mul": [h(pz.mul(pk, z, k)) for z, k in zip(zs, KS)],
        "sum": h(pz.sum_(pk, zs)),
        "add_plain": [h(pz.add_plain(pk, z, m)) for z, m in zip(zs, MS)],
    }
    return out


def main():
    data = {"generator": "tests/golden/gen_golden.py", "cases": [case(1024, 1), case(2048, 0)]}
    path = os.path.join(HERE, "paillier_z_kat.json")
    with open(path, "w") as f:
        json.dump(data, f, indent=1)
    print(path)


if __name__ == "__main__":
    main()

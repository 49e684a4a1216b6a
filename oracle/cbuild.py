"""Build recipe for the oracle's C restatement (test infrastructure only).

gcc -O3 -pthread -shared -fPIC oracle/c/paillier_z_ref.c -> oracle/_build/libpz_ref.so
Portable C11 + unsigned __int128 (gcc on x86-64 and aarch64).
"""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "c", "paillier_z_ref.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpz_ref.so")


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O3", "-std=gnu11", "-pthread", "-shared", "-fPIC", SRC, "-o", tmp]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle C build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))

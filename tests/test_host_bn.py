"""Host big-number code (key generation, batch-inverse root) built with
AddressSanitizer and UndefinedBehaviorSanitizer, every result recomputed
with Python integers.  Needs only g++ (no GPU)."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def host_bn_output(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("hostbn") / "host_bn_test")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
           "-fno-omit-frame-pointer", "-o", exe, os.path.join(HERE, "cpp", "host_bn_test.cpp")]
    build = subprocess.run(cmd, capture_output=True, text=True)
    if build.returncode != 0 and "sanitize" in build.stderr:
        pytest.skip("sanitizer runtime not available: " + build.stderr[-200:])
    assert build.returncode == 0, build.stderr
    res = subprocess.run([exe], capture_output=True, text=True, timeout=600,
                         env=dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="print_stacktrace=1"))
    assert res.returncode == 0, res.stderr[-3000:]
    assert res.stdout.strip().endswith("OK")
    return res.stdout.splitlines()[:-1]


def test_host_bn_matches_python_integers(host_bn_output):
    H = lambda v: int(v, 16)  # noqa: E731
    seen = set()
    for line in host_bn_output:
        op, *f = line.split()
        seen.add(op)
        if op == "add":
            assert H(f[0]) + H(f[1]) == H(f[2])
        elif op == "sub":
            assert H(f[0]) - H(f[1]) == H(f[2])
        elif op == "mul":
            assert H(f[0]) * H(f[1]) == H(f[2])
        elif op == "divmod":
            assert divmod(H(f[0]), H(f[1])) == (H(f[2]), H(f[3]))
        elif op == "shl":
            assert H(f[0]) << int(f[1]) == H(f[2])
        elif op == "shr":
            assert H(f[0]) >> int(f[1]) == H(f[2])
        elif op == "invmod":
            assert H(f[0]) * H(f[2]) % H(f[1]) == 1
        elif op in ("powmod", "montpow"):
            assert pow(H(f[0]), H(f[1]), H(f[2])) == H(f[3])
        elif op == "rootinv":
            x, m, S, got = H(f[0]), H(f[1]), int(f[2]), H(f[3])
            assert got == pow(x, -1, m) * (1 << (32 * S)) % m
    assert seen >= {"add", "sub", "mul", "divmod", "shl", "shr", "invmod", "powmod", "montpow", "rootinv"}

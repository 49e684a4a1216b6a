"""C-ABI boundary checks that need no GPU: the library builds and loads,
exports every symbol the headers declare, host-side key generation agrees
with the oracle, and failures come back as status codes."""

import ctypes

import numpy as np
import pytest

import heu_gb300 as hg
from heu_gb300 import capi
from tests.conftest import oracle_key


def test_library_exports_every_declared_symbol():
    lib = capi.load()
    declared = capi.declared_symbols()
    assert len(declared) >= 30
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, f"undefined C-ABI symbols: {missing}"
    assert set(declared) >= set(capi.SIGNATURES)


def test_host_keygen_matches_oracle_1024():
    k = hg.keygen(1024, 1)
    pk, sk = oracle_key(1024, 1)
    assert (k["n"], k["p"], k["q"], k["h_s"]) == (pk.n, sk.p, sk.q, pk.h_s)


def test_keygen_rejects_bad_sizes():
    lib = capi.load()
    buf = np.zeros(256, np.uint32)
    p = ctypes.c_void_p(buf.ctypes.data)
    assert lib.hg_keygen(1000, 1, p, p, p, p) == capi.HG_ERR_INVALID
    assert b"multiple" in lib.hg_last_error()


def test_null_arguments_are_rejected_without_a_device():
    lib = capi.load()
    assert lib.hg_ctx_create(0, None) == capi.HG_ERR_INVALID
    assert lib.hg_encrypt(None, 1, None, None, None, 4) == capi.HG_ERR_INVALID
    assert lib.hg_key_load(None, 2048, None, None, None, None, 0, None) == capi.HG_ERR_INVALID


def test_context_failure_is_a_status_code_on_a_host_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = capi.load()
    h = ctypes.c_void_p()
    rc = lib.hg_ctx_create(0, ctypes.byref(h))
    assert rc == capi.HG_ERR_CUDA
    assert len(lib.hg_last_error()) > 0


def test_limb_helpers_roundtrip():
    vals = [0, 1, 2 ** 64 + 5, 2 ** 1023 + 17]
    arr = hg.ints_to_limbs(vals, 32)
    assert arr.shape == (4, 32) and arr.dtype == np.uint32
    assert hg.limbs_to_ints(arr) == vals


def test_cpp_spi_adapter_builds_and_generates_the_oracle_key():
    """heu_gb300/cpp/paillier_gb300.h compiles as plain C++17 and its
    KeyGenerator (host only) gives the oracle's key for the same seed."""
    import subprocess

    from tests.conftest import parse_spi_output, spi_test_binary

    exe = spi_test_binary()
    res = subprocess.run([exe, "keygen", "1024", "1"], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    assert res.stdout.strip().endswith("OK")
    got = parse_spi_output(res.stdout)
    pk, sk = oracle_key(1024, 1)
    assert int(got["n"], 16) == pk.n and int(got["p"], 16) == sk.p and int(got["q"], 16) == sk.q
    assert int(got["h_s"], 16) == pk.h_s

import os
import sys

import pytest

# before any CUDA context: every stream its own hardware work queue
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a engine)")
    config.addinivalue_line("markers", "slow: longer CPU-only case")


_KEY_CACHE = {}


def oracle_key(bits, seed):
    """(pk, sk) from the oracle's seeded key generation, cached per session."""
    from oracle import paillier_z as pz

    k = (bits, seed)
    if k not in _KEY_CACHE:
        _KEY_CACHE[k] = pz.keygen(bits, seed)
    return _KEY_CACHE[k]


@pytest.fixture(scope="session")
def gpu_ctx():
    import heu_gb300 as hg

    ctx = hg.Context(0)
    yield ctx
    ctx.close()


_GPU_KEYS = {}


@pytest.fixture(scope="session")
def gpu_key(gpu_ctx):
    """Factory: loaded engine key for (bits, seed) plus the oracle key."""

    def get(bits, seed=0, window=8):
        k = (bits, seed, window)
        if k not in _GPU_KEYS:
            pk, sk = oracle_key(bits, seed)
            _GPU_KEYS[k] = (gpu_ctx.load_key(bits, pk.n, pk.h_s, sk.p, sk.q, table_window=window), pk, sk)
        return _GPU_KEYS[k]

    return get


_SPI_BIN = {}


def spi_test_binary():
    """Builds tests/cpp/spi_test.cpp (the C++ SPI adapter test) with g++
    against the engine library; returns its path."""
    import subprocess

    from heu_gb300 import build as hb
    from heu_gb300 import capi

    capi.load()  # builds the library if it is missing
    if "bin" not in _SPI_BIN:
        out_dir = os.path.join(ROOT, "heu_gb300", "_lib")
        exe = os.path.join(out_dir, "spi_test")
        lib_dir = os.path.dirname(hb.LIB_PATH)
        cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-o", exe,
               os.path.join(ROOT, "tests", "cpp", "spi_test.cpp"), f"-L{lib_dir}", "-lheu_gb300",
               f"-Wl,-rpath,{lib_dir}"]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        _SPI_BIN["bin"] = exe
    return _SPI_BIN["bin"]


def parse_spi_output(text):
    """'name value' lines of spi_test into a dict (hex values as ints where
    they parse)."""
    out = {}
    for line in text.splitlines():
        parts = line.split(" ", 1)
        if len(parts) == 2 and not line.startswith(("FAIL", "audit")):
            out[parts[0]] = parts[1]
    return out

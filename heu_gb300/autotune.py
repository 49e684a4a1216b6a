"""Project autotuner front end: runs the engine's hg_autotune sweep for a key
and persists the chosen configuration per device and key size as JSON.

The sweep (C++, in the engine) times encrypt and scalar mul for both
(threads per ciphertext, limbs per thread) variants and mul windows 2..6,
and CRT decrypt for both mod-p^2 variants and windows 4..7, then applies the
fastest.  The configuration never changes results, only speed.
"""

import ctypes
import fcntl
import json
import os
import tempfile

from heu_gb300 import capi

DEFAULT_CACHE = os.environ.get("HEU_GB300_TUNING",
                               os.path.join(os.path.expanduser("~"), ".cache", "heu_gb300", "tuning.json"))


def device_name(device=0):
    try:
        import torch

        return torch.cuda.get_device_name(device)
    except Exception:
        return f"device{device}"


def tune(key, calib=65536):
    """Run the sweep on `key`; returns (config dict, rates dict)."""
    cfg = capi.KeyConfig()
    rates = (ctypes.c_double * 3)()
    capi.check(key.lib.hg_autotune(key.ctx.handle, key.id, calib, ctypes.byref(cfg), rates))
    return cfg.as_dict(), {"encrypt": rates[0], "mul": rates[1], "decrypt": rates[2]}


def get_config(key):
    cfg = capi.KeyConfig()
    capi.check(key.lib.hg_key_get_config(key.ctx.handle, key.id, ctypes.byref(cfg)))
    return cfg.as_dict()


def set_config(key, config):
    cfg = capi.KeyConfig(**config)
    capi.check(key.lib.hg_key_set_config(key.ctx.handle, key.id, ctypes.byref(cfg)))


def save(config, key_bits, path=DEFAULT_CACHE, device=0, rates=None):
    """Record a key size's configuration in the JSON cache.  The
    read-modify-replace runs under an exclusive lock on a side file, so
    processes and threads saving at once keep each other's entries; the new
    file is written under a unique temporary name and renamed into place."""
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    with open(path + ".lock", "a") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            data = {}
            if os.path.exists(path):
                try:
                    data = json.load(open(path))
                except (OSError, ValueError):
                    data = {}
            entry = {"config": config}
            if rates:
                entry["rates"] = rates
            data.setdefault(device_name(device), {})[str(key_bits)] = entry
            fd, tmp = tempfile.mkstemp(prefix=os.path.basename(path) + ".", suffix=".tmp",
                                       dir=os.path.dirname(path) or ".")
            with os.fdopen(fd, "w") as f:
                json.dump(data, f, indent=1, sort_keys=True)
            os.replace(tmp, path)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


def load(key_bits, path=DEFAULT_CACHE, device=0):
    try:
        data = json.load(open(path))
        return data[device_name(device)][str(key_bits)]["config"]
    except (OSError, ValueError, KeyError):
        return None


def apply_cached(key, path=DEFAULT_CACHE, device=0):
    """Apply a persisted configuration for this key size if one exists."""
    cfg = load(key.key_bits, path, device)
    if cfg:
        set_config(key, cfg)
    return cfg


def tune_and_save(key, calib=65536, path=DEFAULT_CACHE, device=0):
    cfg, rates = tune(key, calib)
    save(cfg, key.key_bits, path, device, rates)
    return cfg, rates

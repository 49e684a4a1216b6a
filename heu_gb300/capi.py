"""ctypes binding of the engine's C-ABI (include/heu_gb300.h).

This is the binding a Python caller (or HEU's pybind layer, through the same
symbols) uses.  Loading fails loudly when the shared library is missing:
there is no CPU fallback.
"""

import ctypes
import os

from heu_gb300 import build as _build

HG_OK = 0
HG_ERR_INVALID = 1
HG_ERR_CT_RANGE = 2
HG_ERR_PT_RANGE = 3
HG_ERR_NOMEM = 4
HG_ERR_CUDA = 5
HG_ERR_NOT_INVERTIBLE = 6
HG_ERR_NO_SECRET = 7
HG_ERR_UNSUPPORTED = 8

ERROR_NAMES = {
    HG_ERR_INVALID: "HG_ERR_INVALID",
    HG_ERR_CT_RANGE: "HG_ERR_CT_RANGE",
    HG_ERR_PT_RANGE: "HG_ERR_PT_RANGE",
    HG_ERR_NOMEM: "HG_ERR_NOMEM",
    HG_ERR_CUDA: "HG_ERR_CUDA",
    HG_ERR_NOT_INVERTIBLE: "HG_ERR_NOT_INVERTIBLE",
    HG_ERR_NO_SECRET: "HG_ERR_NO_SECRET",
    HG_ERR_UNSUPPORTED: "HG_ERR_UNSUPPORTED",
}

_P = ctypes.c_void_p
_SZ = ctypes.c_size_t
_I = ctypes.c_int
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64

# name -> argtypes (every function returns int except where noted)
SIGNATURES = {
    "hg_ctx_create": [_I, ctypes.POINTER(_P)],
    "hg_ctx_destroy": [_P],
    "hg_device_sm_count": [_P],
    "hg_keygen": [_U32, _U64, _P, _P, _P, _P],
    "hg_key_load": [_P, _U32, _P, _P, _P, _P, _I, ctypes.POINTER(_I)],
    "hg_key_free": [_P, _I],
    "hg_ou_keygen": [_U32, _U64, _P, _P, _P, _P, _P, _P, _P, ctypes.POINTER(_I)],
    "hg_ou_key_load": [_P, _U32, _P, _P, _P, _I, _P, _P, _P, _P, _I, ctypes.POINTER(_I)],
    "hg_key_shape": [_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)],
    "hg_encrypt": [_P, _I, _P, _P, _P, _SZ],
    "hg_encrypt_bn": [_P, _I, _P, _P, _P, _P, _SZ],
    "hg_encrypt_zero": [_P, _I, _P, _P, _SZ],
    "hg_randomize": [_P, _I, _P, _P, _SZ],
    "hg_decrypt": [_P, _I, _P, _P, _P, _SZ],
    "hg_decrypt_bn": [_P, _I, _P, _P, _P, _SZ],
    "hg_add": [_P, _I, _P, _P, _P, _SZ],
    "hg_add_plain": [_P, _I, _P, _P, _P, _SZ],
    "hg_sub": [_P, _I, _P, _P, _P, _SZ],
    "hg_sub_plain": [_P, _I, _P, _P, _P, _SZ],
    "hg_plain_sub": [_P, _I, _P, _P, _P, _SZ],
    "hg_mul": [_P, _I, _P, _P, _P, _SZ],
    "hg_mul_bn": [_P, _I, _P, _P, _P, _SZ, _P, _SZ],
    "hg_convert_radix": [_P, _I, _P, _P, _SZ, ctypes.c_uint32, _I],
    "hg_encrypt_encoded": [_P, _I, _I, ctypes.c_int64, _I, _P, _P, _P, _P, _SZ],
    "hg_decrypt_decoded": [_P, _I, _I, ctypes.c_int64, _I, _P, _P, _P, _P, _SZ],
    "hg_dev_encrypt_encoded": [_P, _I, _I, ctypes.c_int64, _I, _P, _P, _P, _P, _SZ, _P],
    "hg_dev_decrypt_decoded": [_P, _I, _I, ctypes.c_int64, _I, _P, _P, _P, _P, _SZ, _P],
    "hg_negate": [_P, _I, _P, _P, _SZ],
    "hg_sum": [_P, _I, _P, _SZ, _P],
    "hg_to_mont": [_P, _I, _P, _P, _SZ],
    "hg_from_mont": [_P, _I, _P, _P, _SZ],
    "hg_dev_encrypt": [_P, _I, _P, _P, _P, _SZ, _P],
    "hg_dev_decrypt": [_P, _I, _P, _P, _P, _SZ, _P],
    "hg_dev_add": [_P, _I, _P, _P, _P, _SZ, _P],
    "hg_dev_mul": [_P, _I, _P, _P, _P, _SZ, _P],
    "hg_dev_mul_bn": [_P, _I, _P, _P, _P, _SZ, _P, _SZ, _P],
    "hg_dev_sum": [_P, _I, _P, _SZ, _P, _P],
    "hg_dev_encrypt_zero": [_P, _I, _P, _P, _SZ, _P],
    "hg_dev_randomize": [_P, _I, _P, _P, _SZ, _P],
    "hg_dev_add_plain": [_P, _I, _P, _P, _P, _SZ, _P],
    "hg_dev_sub_plain": [_P, _I, _P, _P, _P, _SZ, _P],
    "hg_dev_plain_sub": [_P, _I, _P, _P, _P, _SZ, _P],
    "hg_dev_sub": [_P, _I, _P, _P, _P, _SZ, _P],
    "hg_dev_negate": [_P, _I, _P, _P, _SZ, _P],
    "hg_dev_sum_noalloc": [_P, _I, _P, _SZ, _P, _P],
    "hg_dev_check": [_P],
    "hg_serialize_bound": [_P, _I, _SZ, ctypes.POINTER(_SZ)],
    "hg_serialize": [_P, _I, _P, _SZ, _SZ, _I, _I, _P, _SZ, ctypes.POINTER(_SZ)],
    "hg_deserialize": [_P, _I, _P, _SZ, _I, _P, _SZ, ctypes.POINTER(_SZ), ctypes.POINTER(_SZ), ctypes.POINTER(_I)],
    "hg_dev_serialize": [_P, _I, _P, _SZ, _SZ, _I, _I, _P, _SZ, ctypes.POINTER(_SZ), _P],
    "hg_dev_deserialize": [_P, _I, _P, _SZ, _I, _P, _SZ, ctypes.POINTER(_SZ), ctypes.POINTER(_SZ),
                           ctypes.POINTER(_I), _P],
    "hg_bucket_sum": [_P, _I, _P, _SZ, _SZ, _P, _SZ, _I, _I, _P],
    "hg_dev_bucket_sum": [_P, _I, _P, _SZ, _SZ, _P, _SZ, _I, _I, _P, _P],
    "hg_matmul": [_P, _I, _P, _SZ, _SZ, _P, _SZ, _P],
    "hg_dev_matmul": [_P, _I, _P, _SZ, _SZ, _P, _SZ, _P, _P],
    "hg_matmul_bn": [_P, _I, _P, _SZ, _SZ, _P, _P, _SZ, _SZ, _P],
    "hg_dev_matmul_bn": [_P, _I, _P, _SZ, _SZ, _P, _P, _SZ, _SZ, _P, _P],
    "hg_key_get_config": [_P, _I, _P],
    "hg_key_set_config": [_P, _I, _P],
    "hg_autotune": [_P, _I, _SZ, _P, _P],
    "hg_batch_create": [_P, ctypes.POINTER(_P)],
    "hg_batch_destroy": [_P],
    "hg_batch_add": [_P, _I, _I, _SZ, _P, _P, _P, _P, _I],
    "hg_batch_clear": [_P],
    "hg_batch_set_variant": [_P, _I],
    "hg_batch_run": [_P, _P, _I],
    "hg_batch_wait": [_P, _P],
    "hg_server_create": [_P, _P, ctypes.POINTER(_P)],
    "hg_server_destroy": [_P],
    "hg_server_store": [_P, _I, _P, _SZ, ctypes.POINTER(_U64)],
    "hg_server_release": [_P, _U64],
    "hg_server_submit": [_P, _P, ctypes.POINTER(_U64)],
    "hg_server_wait": [_P, _U64, ctypes.POINTER(ctypes.c_double)],
    "hg_server_stats": [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64), ctypes.POINTER(_SZ), ctypes.POINTER(_SZ)],
    "hg_probe_serve_load": [_P, _P, _P, _P, _P, ctypes.POINTER(ctypes.c_double)],
    "hg_probe_server_trace": [_P, _I, _P, _SZ, ctypes.POINTER(_SZ)],
    "hg_probe_mac_peak": [_I, _I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)],
    "hg_probe_launch_count": [ctypes.POINTER(_U64)],
    "hg_probe_set_alloc_limit": [_SZ, ctypes.POINTER(_SZ)],
    "hg_probe_host_copy": [_I, _P, ctypes.c_size_t, _I, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)],
}

_lib = None

HG_OP_ENCRYPT, HG_OP_DECRYPT, HG_OP_ADD, HG_OP_MUL, HG_OP_SUM = 0, 1, 2, 3, 4
HG_CODEC_PLAIN_I64, HG_CODEC_PLAIN_F64, HG_CODEC_BATCH_I64, HG_CODEC_BATCH_F64 = 1, 2, 3, 4
HG_JOB_NONNEG = 1
HG_BATCH_PER_KEY = -1


class ServerConfig(ctypes.Structure):
    """hg_server_config"""

    _fields_ = [("budget_bytes", ctypes.c_size_t), ("slots", ctypes.c_int), ("max_batch_elems", ctypes.c_size_t),
                ("variant", ctypes.c_int), ("batch_us", ctypes.c_double), ("slice_us", ctypes.c_double),
                ("policy", ctypes.c_int), ("express_us", ctypes.c_double), ("express_share", ctypes.c_double),
                ("express_len", ctypes.c_size_t)]


class Request(ctypes.Structure):
    """hg_request"""

    _fields_ = [("key_id", ctypes.c_int), ("op", ctypes.c_int), ("count", ctypes.c_size_t),
                ("in0", ctypes.c_void_p), ("in1", ctypes.c_void_p), ("h0", ctypes.c_uint64),
                ("h1", ctypes.c_uint64), ("out", ctypes.c_void_p), ("aux", ctypes.c_void_p)]


class LoadSpec(ctypes.Structure):
    """hg_load_spec"""

    _fields_ = [("key_ids", ctypes.c_void_p), ("nkeys", ctypes.c_int), ("handles", ctypes.c_void_p),
                ("rate", ctypes.c_double), ("nreq", ctypes.c_size_t), ("len_min", ctypes.c_size_t),
                ("len_max", ctypes.c_size_t), ("op_weights", ctypes.c_double * 5), ("seed", ctypes.c_uint64),
                ("m_host", ctypes.c_void_p), ("r_host", ctypes.c_void_p), ("k_host", ctypes.c_void_p),
                ("sink", ctypes.c_void_p), ("phases", ctypes.c_void_p)]


class KeyConfig(ctypes.Structure):
    """hg_key_config"""

    _fields_ = [("variant", ctypes.c_int), ("dec_variant", ctypes.c_int), ("mul_window", ctypes.c_int),
                ("dec_window", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class HgError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {message}")
        self.code = code


def lib_path():
    return _build.LIB_PATH


def load(build_if_missing=True):
    """Load the C-ABI library (building it in-tree first if asked)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"heu_gb300 native library not found at {path}; run heu_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _I
    lib.hg_last_error.argtypes = []
    lib.hg_last_error.restype = ctypes.c_char_p
    _lib = lib
    return lib


def check(code):
    if code != HG_OK:
        msg = _lib.hg_last_error().decode(errors="replace") if _lib is not None else ""
        raise HgError(code, msg)


def declared_symbols():
    """Function names declared in the headers under include/."""
    import glob
    import re

    names = set()
    for header_path in glob.glob(os.path.join(os.path.dirname(_build.HERE), "include", "*.h")):
        text = open(header_path).read()
        names.update(re.findall(r"^\s*(?:int|const char\*)\s+(hg_\w+)\s*\(", text, re.M))
    return sorted(names)


def launch_count():
    """Engine kernels launched by this process so far."""
    v = _U64()
    check(load().hg_probe_launch_count(ctypes.byref(v)))
    return v.value


def mac_peak(device=0, pattern=0):
    """Measured integer MAC/s of the device for the given instruction pattern."""
    lib = load()
    v, secs = ctypes.c_double(), ctypes.c_double()
    rc = lib.hg_probe_mac_peak(device, pattern, ctypes.byref(v), ctypes.byref(secs))
    if rc != 0:
        raise HgError(rc, "MAC peak probe failed")
    return v.value

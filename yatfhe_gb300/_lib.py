"""ctypes binding of the C ABI in include/yatfhe_gb300.h.

The library is loaded from yatfhe_gb300/_build/ (built in-tree by yatfhe_gb300/build.py).
There is no fallback: if the shared library is missing or cannot be loaded, every entry
point raises.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

from .params import PbsParams

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libyatfhe_gb300.so"

YG_OK = 0
_ERRORS = {-1: ValueError, -2: RuntimeError, -3: OSError, -4: MemoryError, -5: RuntimeError}


class YgParams(ctypes.Structure):
    _fields_ = [(f, ctypes.c_int) for f in ("n", "N", "k", "radix_bits", "l_approx", "ks_radix_bits", "ks_level",
                                            "torus_bits")]

    @classmethod
    def of(cls, p: PbsParams) -> "YgParams":
        return cls(p.n, p.N, p.k, p.radix_bits, p.l_approx, p.ks_radix_bits, p.ks_level, p.torus_bits)


_vp = ctypes.c_void_p
_SIGNATURES = {
    "yg_last_error": (ctypes.c_char_p, []),
    "yg_ctx_create": (ctypes.c_int, [ctypes.POINTER(YgParams), ctypes.c_int, ctypes.POINTER(_vp)]),
    "yg_ctx_destroy": (None, [_vp]),
    "yg_key_load_bsk_file": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.POINTER(_vp)]),
    "yg_key_upload_bsk_ntt": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(_vp)]),
    "yg_key_set_ksk": (ctypes.c_int, [_vp, _vp]),
    "yg_key_destroy": (None, [_vp]),
    "yg_key_device_bytes": (ctypes.c_size_t, [_vp]),
    "yg_pbs": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, _vp, _vp]),
    "yg_pbs_host": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, _vp, _vp]),
    "yg_blind_rotate": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "yg_keyswitch": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "yg_blind_rotate_extract": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "yg_blind_rotate_acc": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "yg_key_create_ksk_only": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "yg_pbs_noalloc": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, _vp, _vp]),
    "yg_pbs_noalloc_max_count": (ctypes.c_size_t, [_vp]),
    "yg_probe_int32_rate": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
}

_lib = None
_lock = threading.Lock()


def exported_symbols() -> list[str]:
    return sorted(_SIGNATURES)


def lib() -> ctypes.CDLL:
    """The loaded library; raises if it was not built."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(f"{LIB_PATH} is missing: run yatfhe_gb300.build.build() (nvcc, sm_103a) first")
            l = ctypes.CDLL(str(LIB_PATH))
            for name, (res, args) in _SIGNATURES.items():
                fn = getattr(l, name)
                fn.restype = res
                fn.argtypes = args
            _lib = l
        return _lib


def check(rc: int) -> None:
    if rc != YG_OK:
        msg = lib().yg_last_error().decode(errors="replace")
        raise _ERRORS.get(rc, RuntimeError)(msg or f"yatfhe_gb300 error {rc}")

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
LAYOUT_CHANNEL = 0      # YG_LAYOUT_CHANNEL
LAYOUT_CHANNEL_ROW = 1  # YG_LAYOUT_CHANNEL_ROW
LAYOUT_ROW_CLUSTER = 2  # YG_LAYOUT_ROW_CLUSTER
LAYOUT_CHANNEL_CLUSTER = 3  # YG_LAYOUT_CHANNEL_CLUSTER
_ERRORS = {-1: ValueError, -2: RuntimeError, -3: OSError, -4: MemoryError, -5: RuntimeError}


class YgParams(ctypes.Structure):
    _fields_ = [(f, ctypes.c_int) for f in ("n", "N", "k", "radix_bits", "l_approx", "ks_radix_bits", "ks_level",
                                            "torus_bits")]

    @classmethod
    def of(cls, p: PbsParams) -> "YgParams":
        return cls(p.n, p.N, p.k, p.radix_bits, p.l_approx, p.ks_radix_bits, p.ks_level, p.torus_bits)


class ServerConfig(ctypes.Structure):
    _fields_ = [("key_budget_bytes", ctypes.c_size_t), ("max_batch", ctypes.c_int), ("max_inflight", ctypes.c_int),
                ("max_tenants", ctypes.c_int), ("latency_batch_max", ctypes.c_int)]


class ServerCounters(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in ("key_hits", "key_misses", "refill_bytes", "batches", "requests_done",
                                               "ciphertexts_done")] + [("key_slots", ctypes.c_int),
                                                                       ("latency_batches", ctypes.c_uint64)]


class RequestTimes(ctypes.Structure):
    _fields_ = [(f, ctypes.c_double) for f in ("t_submit", "t_start", "t_done")]


class TraceConfig(ctypes.Structure):
    _fields_ = [("requests", ctypes.c_int), ("warmup", ctypes.c_int), ("rate", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("zipf_s", ctypes.c_double), ("zipf_seed", ctypes.c_uint64),
                ("tenants", ctypes.c_int), ("max_count", ctypes.c_int), ("queue_max", ctypes.c_int),
                ("h_pool", ctypes.c_void_p), ("h_expect", ctypes.c_void_p), ("slo_ms", ctypes.c_double)]


class Latency(ctypes.Structure):
    _fields_ = [(f, ctypes.c_double) for f in ("mean_ms", "p50_ms", "p90_ms", "p99_ms", "p999_ms", "max_ms")]


class TraceResult(ctypes.Structure):
    _fields_ = [("served", ctypes.c_int), ("shed", ctypes.c_int), ("mismatched_requests", ctypes.c_int),
                ("seconds", ctypes.c_double), ("requests_per_s", ctypes.c_double),
                ("ciphertexts_per_s", ctypes.c_double), ("offered_rate", ctypes.c_double),
                ("sojourn", Latency), ("queue", Latency), ("service", Latency),
                ("key_hits", ctypes.c_uint64), ("key_misses", ctypes.c_uint64), ("refill_bytes", ctypes.c_uint64),
                ("batches", ctypes.c_uint64), ("hit_rate", ctypes.c_double),
                ("slo_ms", ctypes.c_double), ("slo_violation_rate", ctypes.c_double),
                ("slo_violation_rate_100", ctypes.c_double), ("slo_violation_rate_300", ctypes.c_double),
                ("slo_violation_rate_500", ctypes.c_double), ("tenant_fairness_jain", ctypes.c_double),
                ("peak_queue_depth", ctypes.c_int), ("load_concurrency_peak", ctypes.c_int),
                ("load_concurrency_mean", ctypes.c_double), ("latency_batches", ctypes.c_uint64)]


_vp = ctypes.c_void_p
_SIGNATURES = {
    "yg_last_error": (ctypes.c_char_p, []),
    "yg_ctx_create": (ctypes.c_int, [ctypes.POINTER(YgParams), ctypes.c_int, ctypes.POINTER(_vp)]),
    "yg_ctx_destroy": (None, [_vp]),
    "yg_key_load_bsk_file": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.POINTER(_vp)]),
    "yg_key_upload_bsk_ntt": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(_vp)]),
    "yg_key_upload_wwl24_ntt": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.POINTER(_vp)]),
    "yg_key_load_wwl24_file": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.POINTER(_vp)]),
    "yg_key_upload_lazy": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.POINTER(_vp)]),
    "yg_key_load_lazy_file": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.POINTER(_vp)]),
    "yg_key_upload_group": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_vp)]),
    "yg_keygen_from_samples": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.POINTER(_vp)]),
    "yg_keygen": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.POINTER(_vp)]),
    "yg_draw_keygen_samples": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp,
                                              _vp, _vp]),
    "yg_encrypt_lwe": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int,
                                      _vp, _vp]),
    "yg_encrypt_lwe_from_samples": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp, _vp]),
    "yg_encrypt_rlwe_ntt": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint32,
                                           ctypes.c_int, _vp, _vp]),
    "yg_encrypt_rlwe_ntt_from_samples": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp, _vp]),
    "yg_crt_key_upload": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, ctypes.POINTER(_vp)]),
    "yg_crt_blind_rotate": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, _vp, _vp]),
    "yg_crt_key_device_bytes": (ctypes.c_size_t, [_vp]),
    "yg_crt_key_destroy": (None, [_vp]),
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
    "yg_plan_create": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp, _vp, ctypes.c_int, _vp, ctypes.c_int,
                                      ctypes.POINTER(_vp)]),
    "yg_plan_set_launch": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "yg_plan_run": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "yg_plan_destroy": (None, [_vp]),
    "yg_ctas_per_sm": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "yg_ctx_set_launch": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "yg_server_create": (ctypes.c_int, [_vp, ctypes.POINTER(ServerConfig), ctypes.POINTER(_vp)]),
    "yg_server_add_tenant": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp]),
    "yg_server_start": (ctypes.c_int, [_vp]),
    "yg_server_submit": (ctypes.c_int64, [_vp, ctypes.c_int, _vp, _vp, ctypes.c_int]),
    "yg_server_wait": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(RequestTimes)]),
    "yg_server_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ServerCounters)]),
    "yg_server_destroy": (None, [_vp]),
    "yg_server_run_trace": (ctypes.c_int, [_vp, ctypes.POINTER(TraceConfig), ctypes.POINTER(TraceResult)]),
    "yg_probe_int32_rate": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "yg_wait_timeouts": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_uint64)]),
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

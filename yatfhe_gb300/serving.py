"""Python view of the serving loop (yg_server_*): tenants, requests and whole traces.

    srv = Server(ctx, key_budget_bytes=4e9, max_batch=4096)
    srv.add_tenant(0, key0, lut)            # before start
    srv.start()
    rid = srv.submit(0, h_in, h_out)        # pinned int32 arrays [count, n+1]
    times = srv.wait(rid)
    result = srv.run_trace(pool, expect=..., requests=..., rate=...)
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .api import BootstrapKey, Context


def _latency(l) -> dict:
    return {k: getattr(l, k) for k, _ in _lib.Latency._fields_}


class Server:
    def __init__(self, ctx: Context, key_budget_bytes: float, max_batch: int = 4096, max_inflight: int = 2,
                 max_tenants: int = 1024, latency_batch_max: int = 0):
        cfg = _lib.ServerConfig(int(key_budget_bytes), max_batch, max_inflight, max_tenants, latency_batch_max)
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().yg_server_create(ctx.handle, ctypes.byref(cfg), ctypes.byref(h)))
        self.ctx, self._h, self.max_batch = ctx, h, max_batch

    def add_tenant(self, tenant: int, key: BootstrapKey, lut: np.ndarray) -> None:
        v = np.ascontiguousarray(lut, np.int64)
        _lib.check(_lib.lib().yg_server_add_tenant(self._h, tenant, key.handle, ctypes.c_void_p(v.ctypes.data)))

    def start(self) -> None:
        _lib.check(_lib.lib().yg_server_start(self._h))

    def submit(self, tenant: int, h_in, h_out, count: int | None = None) -> int:
        count = len(h_in) if count is None else count
        rid = _lib.lib().yg_server_submit(self._h, tenant, ctypes.c_void_p(_addr(h_in)),
                                          ctypes.c_void_p(_addr(h_out)), count)
        if rid <= 0:
            _lib.check(int(rid))
        return rid

    def wait(self, rid: int, timeout_ms: int = 600000) -> dict:
        t = _lib.RequestTimes()
        _lib.check(_lib.lib().yg_server_wait(self._h, rid, timeout_ms, ctypes.byref(t)))
        return {"t_submit": t.t_submit, "t_start": t.t_start, "t_done": t.t_done}

    def counters(self) -> dict:
        c = _lib.ServerCounters()
        _lib.check(_lib.lib().yg_server_stats(self._h, ctypes.byref(c)))
        return {k: getattr(c, k) for k, _ in _lib.ServerCounters._fields_}

    def run_trace(self, pool, expect=None, *, requests: int, rate: float, warmup: int = 0, seed: int = 1,
                  zipf_s: float = 1.1, zipf_seed: int = 20260816, max_count: int = 256, queue_max: int = 0,
                  slo_ms: float = 100.0) -> dict:
        """pool / expect: pinned int32 arrays [tenants, max_count, n+1] (expect may be None)."""
        tenants = pool.shape[0]
        cfg = _lib.TraceConfig(requests, warmup, float(rate), seed, float(zipf_s), zipf_seed, tenants, max_count,
                               queue_max, ctypes.c_void_p(_addr(pool)),
                               None if expect is None else ctypes.c_void_p(_addr(expect)), float(slo_ms))
        r = _lib.TraceResult()
        _lib.check(_lib.lib().yg_server_run_trace(self._h, ctypes.byref(cfg), ctypes.byref(r)))
        out = {k: getattr(r, k) for k, _ in _lib.TraceResult._fields_ if k not in ("sojourn", "queue", "service")}
        out.update(sojourn=_latency(r.sojourn), queue=_latency(r.queue), service=_latency(r.service))
        return out

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.lib().yg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _addr(a) -> int:
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data

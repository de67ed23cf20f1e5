#!/usr/bin/env python
"""Benchmark: bootstraps/s of the GINX/MP21 programmable bootstrap on GB300.

One step = one full bootstrap (modulus switch, blind rotation, sample extraction, key
switch) of a batch of ciphertexts under one key, through the C ABI.  Default workload:
the TORUS=32 set (n=630, N=1024, B=2^7, l=3, KS 2^2 x 8) batched at 65,536 ciphertexts.

Printed JSON line (rank 0): value = whole-job bootstraps/s with inputs resident in HBM
(CUDA events on the launching stream, max over ranks); e2e = the same through the
host-buffer entry point (yg_pbs_host: pinned host -> device copy, bootstrap, copy back);
roofline of the dominant kernel (blind rotation) against the measured 32-bit
multiply-add rate; cpu_baseline = the CPU oracle on the host cores on a bounded sample,
which also checks the sampled GPU outputs bit for bit.  Unless --no-extras, the line also
carries the plain per-call form, a batch-size sweep and the other workloads under
"workloads": the TORUS=56 set at 16,384 ciphertexts, the 32-tenant mixed-parameter batch
in one CUDA graph, and the 128-tenant serving trace (p50/p99 at 50-100 % of peak).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--params t32_n1024|t56_n2048]
                  [--count C] [--impl ours|reference] [--workload batch|multi_tenant|serving|serving_lazy|encrypt|crt|lone]
Multi-GPU: one process per GPU (torchrun); every rank bootstraps its own batch (weak
scaling, no data-path collective).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time
import traceback
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "bootstraps/s"
L2_BYTES = 129 * 2**20
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--params", default="t32_n1024")
    ap.add_argument("--count", type=int, default=0, help="ciphertexts per step (default 65536 / 16384)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch", choices=["batch", "multi_tenant", "serving", "serving_lazy",
                                                                  "encrypt", "crt", "lone"])
    ap.add_argument("--no-extras", action="store_true", help="skip the per-call / sweep legs and other workloads")
    ap.add_argument("--cpu-sample", type=int, default=0, help="ciphertexts in the CPU baseline sample")
    ap.add_argument("--per-cta", type=int, default=0, help="fix ciphertexts per CTA (skips the autotuner)")
    ap.add_argument("--ctas-per-sm", type=int, default=0, help="with --per-cta: persistent CTAs per SM (0 = off)")
    ap.add_argument("--layout", type=int, default=0,
                    help="with --per-cta: 0 = team per channel, 1 = per channel and row, 2 = two-CTA row cluster")
    ap.add_argument("--retune", action="store_true", help="re-measure launch shapes instead of the cached choice")
    ap.add_argument("--serving-requests", type=int, default=800, help="measured requests per offered rate")
    ap.add_argument("--serving-fractions", default="0.5,0.6,0.7,0.8,0.9,1.0", help="offered rates / peak")
    ap.add_argument("--serving-max-batch", type=int, default=304, help="ciphertexts per serving batch")
    ap.add_argument("--serving-inflight", type=int, default=2, help="serving batches on the GPU at once")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def synthetic_keys(p, seed):
    """Seeded synthetic keys with the shapes of a real key set: NTT-domain BSK words are
    uniform mod q (as a real key's are: its masks are sampled uniformly in that domain), KSK
    words uniform mod 2^32 (as real masks are)."""
    rng = np.random.default_rng(seed)
    bsk = rng.integers(0, p.q_ntt, size=p.bsk_ntt_words, dtype=np.uint64)
    ksk = rng.integers(-(1 << 31), 1 << 31, size=p.ksk_words, dtype=np.int64).astype(np.int32)
    return bsk, ksk


def synthetic_lwe(p, count, seed):
    """count LWE ciphertexts with uniform 32-bit words (what encryptions look like)."""
    rng = np.random.default_rng(seed)
    return rng.integers(-(1 << 31), 1 << 31, size=(count, p.n + 1), dtype=np.int64).astype(np.int32)


def workload_lut(p, seed=5):
    """TORUS=32: the sign bootstrap's constant test polynomial; TORUS=56: a random 4-bit
    lookup table in the padded box layout (messages m in 0..15 -> LUT[m])."""
    from yatfhe_gb300 import lut as lutmod

    if p.torus_bits == 32:
        return lutmod.sign_lut(p.N, p.torus_bits)
    table = np.random.default_rng(seed).integers(0, 16, 16)
    return lutmod.padded_message_lut(p.N, p.torus_bits, table)


def ops_per_bootstrap(p):
    """Multiply-class 32-bit operations per bootstrap: 9 per mod-q multiplication (3 RNS
    channels x 3 for a Shoup word multiply) over the blind rotation's modmul count
    M = n [2l (N/2) log2 N + 4 l N + 2 (N/2) log2 N], plus the key switch's k N t (n+1) MACs."""
    logN = int(np.log2(p.N))
    L = p.l_approx
    M = p.n * (2 * L * (p.N // 2) * logN + 4 * L * p.N + 2 * (p.N // 2) * logN)
    ks = p.k * p.N * p.ks_level * (p.n + 1)
    return 9 * M, ks


def zipf_counts(s: float, n: int, draws: int, seed: int) -> np.ndarray:
    """Per-rank counts of `draws` Zipf(s) samples over n ranks, drawn by inverse CDF as the
    reference's ZipfDistribution does (yatfhe/include/yautil/zipf.h:47-87: harmonic
    normalisation, lower_bound of a uniform draw, rank clamped to n-1); numpy's generator
    supplies the uniforms."""
    k = np.arange(1, n + 1, dtype=np.float64)
    w = k ** -s
    cdf = np.cumsum(w / w.sum())
    cdf[-1] = 1.0
    u = np.random.default_rng(seed).random(draws)
    r = np.minimum(np.searchsorted(cdf, u, side="left"), n - 1)
    return np.bincount(r, minlength=n)


def measured_peaks() -> dict:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        return json.loads(f.read_text())
    return {}


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        low = sorted(sm)[len(sm) // 10] if sm else None
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_p10_mhz": low, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def traffic_from_profiles(kernel: str, workload: str):
    """dram bytes per launch recorded in profiles/<kernel>_<workload>.md ('traffic_bytes_per_launch: X')."""
    f = ROOT / "profiles" / f"{kernel}_{workload}.md"
    if not f.exists():
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", f.read_text())
    return float(m.group(1)) if m else None


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_cpu_baseline(p, bsk, ksk, lwe, lut, sample, threads, latency=False):
    """The CPU oracle (plain-C restatement of the reference path) on `sample` ciphertexts:
    (outputs, bootstraps/s, seconds, and with `latency` the milliseconds of one bootstrap on
    one thread, else None)."""
    from oracle.oracle import Restatement

    ora = Restatement(p)
    ora.set_bsk_ntt(bsk)
    ora.set_ksk(ksk)
    t0 = time.perf_counter()
    out = ora.pbs(lwe[:sample], lut, threads=threads)
    dt = time.perf_counter() - t0
    lat = None
    if latency:
        t1 = time.perf_counter()
        ora.pbs(lwe[:1], lut, threads=1)
        lat = (time.perf_counter() - t1) * 1e3
    return out, sample / dt, dt, lat


def params_config(p) -> dict:
    return {"n": p.n, "N": p.N, "k": p.k, "B": 1 << p.radix_bits, "l": p.l_approx, "ks_base": 1 << p.ks_radix_bits,
            "ks_t": p.ks_level, "torus_bits": p.torus_bits}


# ------------------------------------------------------------------------------ one key, one batch

class BatchRun:
    """One parameter set, one synthetic key, `count` resident ciphertexts; times the
    blind-rotation(+extract) and key-switch launches of each step with CUDA events."""

    def __init__(self, p, count, dev, seed, per_cta=0, ctas_per_sm=0, retune=False, layout=0):
        import torch

        from yatfhe_gb300 import _lib, api

        self.p, self.count, self.dev = p, count, dev
        self.L = _lib.lib()
        self.bsk, self.ksk = synthetic_keys(p, seed)
        self.lwe = synthetic_lwe(p, count, seed + 1)
        self.lut = workload_lut(p)
        self.ctx = api.Context(p, dev)
        t0 = time.perf_counter()
        self.key = api.BootstrapKey.from_ntt_words(self.ctx, self.bsk).set_ksk(self.ksk)
        self.key_upload_s = time.perf_counter() - t0
        self.stream = torch.cuda.Stream(device=dev)
        self.sh = ctypes.c_void_p(self.stream.cuda_stream)
        self.d_in = torch.from_numpy(self.lwe).to(f"cuda:{dev}")
        self.d_lut = torch.from_numpy(self.lut).to(f"cuda:{dev}")
        if per_cta:
            api.set_launch(self.ctx, per_cta, ctas_per_sm, layout)
            self.tuning = {"choice": {"layout": layout, "per_cta": per_cta, "ctas_per_sm": ctas_per_sm},
                           "fixed": True}
        else:
            from yatfhe_gb300 import autotune

            self.tuning = autotune.tune(self.ctx, self.key, self.d_lut, use_cache=not retune)
        self.d_big = torch.empty((count, p.k * p.N + 1), dtype=torch.int32, device=f"cuda:{dev}")
        self.d_out = torch.empty_like(self.d_in)
        torch.cuda.synchronize(dev)

    def step(self, ev=None):
        from yatfhe_gb300 import _lib

        if ev:
            ev[0].record(self.stream)
        _lib.check(self.L.yg_blind_rotate_extract(self.ctx.handle, self.key.handle, ctypes.c_void_p(self.d_in.data_ptr()),
                                                  ctypes.c_void_p(self.d_lut.data_ptr()),
                                                  ctypes.c_void_p(self.d_big.data_ptr()), self.count, self.sh))
        if ev:
            ev[1].record(self.stream)
        _lib.check(self.L.yg_keyswitch(self.ctx.handle, self.key.handle, ctypes.c_void_p(self.d_big.data_ptr()),
                                       ctypes.c_void_p(self.d_out.data_ptr()), self.count, self.sh))
        if ev:
            ev[2].record(self.stream)

    def timed(self, steps, warmup, barrier=None, clocks=None):
        import torch

        for _ in range(warmup):
            self.step()
        self.stream.synchronize()
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if barrier:
            barrier()
        if clocks:
            clocks.start()
        start.record(self.stream)
        for k in range(steps):
            self.step(evs[k])
        end.record(self.stream)
        self.stream.synchronize()
        if barrier:
            barrier()
        clock_info = clocks.stop() if clocks else None
        return {"total_ms": start.elapsed_time(end), "br_ms": [e[0].elapsed_time(e[1]) for e in evs],
                "ks_ms": [e[1].elapsed_time(e[2]) for e in evs], "clocks": clock_info}

    def roofline(self, br_ms, int32_peak_tops, workload):
        p = self.p
        br_ops, _ = ops_per_bootstrap(p)
        br_avg_s = statistics.mean(br_ms) / 1e3
        achieved = br_ops * self.count / br_avg_s / 1e12
        bsk_alg = p.n * p.l_approx * (p.k + 1) ** 2 * p.N * 8
        io_alg = self.count * ((p.n + 1) + (p.k * p.N + 1)) * 4
        hbm = measured_peaks().get("hbm_gbs", FALLBACK_HBM_GBS)
        hbm_achieved = (bsk_alg + io_alg) / br_avg_s / 1e9
        return {
            "bound": "int32", "kernel": "blind_rotate_kernel", "achieved": achieved, "peak": int32_peak_tops,
            "unit": "TOP/s", "frac": achieved / int32_peak_tops,
            "peak_source": "measured: yg_probe_int32_rate (32-bit IMAD chains, all SMs)",
            "ops_per_bootstrap": br_ops, "launch_ms": statistics.mean(br_ms),
            "traffic": traffic_from_profiles("blind_rotate_kernel", workload),
            "hbm_view": {"algorithmic_bytes_per_launch": bsk_alg + io_alg, "achieved_gbs": hbm_achieved,
                         "peak_gbs": hbm, "frac": hbm_achieved / hbm,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs" if measured_peaks() else "fallback 6.8 TB/s"},
        }


def int32_peak(dev) -> float:
    from yatfhe_gb300 import _lib

    rate = ctypes.c_double()
    _lib.check(_lib.lib().yg_probe_int32_rate(dev, ctypes.byref(rate)))
    return rate.value / 1e12


# ------------------------------------------------------------------------------ other workloads

def leg_t56(dev, steps=2, warmup=1, count=16384):
    """TORUS=56 set (n=750, N=2048, B=2^10, l=4, KS 2^3 x 10), 16,384 ciphertexts, random
    4-bit LUT."""
    from yatfhe_gb300.params import T56_N2048

    run = BatchRun(T56_N2048, count, dev, seed=0x5EED0003)
    t = run.timed(steps, warmup)
    workload = f"t56_n2048_batch{count}"
    return {"workload": workload, "params": params_config(T56_N2048), "ciphertexts_per_step": count,
            "value": count * steps / (t["total_ms"] / 1e3), "unit": "bootstraps/s", "steps": steps,
            "ms_per_step": t["total_ms"] / steps, "keyswitch_ms": statistics.mean(t["ks_ms"]),
            "roofline": run.roofline(t["br_ms"], int32_peak(dev), workload), "launch_shape": run.tuning}


def leg_wwl24(dev, steps=2, warmup=1, count=16384):
    """WWL+24 keys on the reference's default TORUS=32 set (n=680, N=2048, B=2^4, lApprox=4,
    s2 key with l=8 levels, KS 2^2 x 16): seeded synthetic half key (cPrime rows and s2 key
    uniform mod q, like a real key's NTT-domain words), uploaded through
    yg_key_upload_wwl24_ntt (the GINX rows derived on the GPU, then the usual conversion),
    then `count` bootstraps per step.  Reports the upload's wall time and host bytes beside
    the GINX key's, and the throughput on the derived key."""
    import torch

    from yatfhe_gb300 import _lib, api
    from yatfhe_gb300.params import WWL24_T32_N2048 as p

    rng = np.random.default_rng(0x5EED0005)
    row = (p.k + 1) * p.N
    cprime = rng.integers(0, p.q_ntt, size=p.n * p.l_approx * row, dtype=np.uint64)
    s2 = rng.integers(0, p.q_ntt, size=p.l * row, dtype=np.uint64)
    ksk = rng.integers(-(1 << 31), 1 << 31, size=p.ksk_words, dtype=np.int64).astype(np.int32)
    ctx = api.Context(p, dev)
    uploads = []
    for _ in range(3):  # the first call also pays one-time setup; the best of three is reported
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        key = api.BootstrapKey.from_wwl24_words(ctx, cprime, s2)
        uploads.append(time.perf_counter() - t0)
        key.close()
    key = api.BootstrapKey.from_wwl24_words(ctx, cprime, s2).set_ksk(ksk)
    lwe = synthetic_lwe(p, count, 0x5EED0006)
    lut = workload_lut(p)
    d_in = torch.from_numpy(lwe).to(f"cuda:{dev}")
    d_lut = torch.from_numpy(lut).to(f"cuda:{dev}")
    d_big = torch.empty((count, p.k * p.N + 1), dtype=torch.int32, device=f"cuda:{dev}")
    d_out = torch.empty_like(d_in)
    from yatfhe_gb300 import autotune

    tuning = autotune.tune(ctx, key, d_lut)
    L = _lib.lib()
    stream = torch.cuda.Stream(device=dev)
    sh = ctypes.c_void_p(stream.cuda_stream)

    def step():
        _lib.check(L.yg_blind_rotate_extract(ctx.handle, key.handle, ctypes.c_void_p(d_in.data_ptr()),
                                             ctypes.c_void_p(d_lut.data_ptr()), ctypes.c_void_p(d_big.data_ptr()),
                                             count, sh))
        _lib.check(L.yg_keyswitch(ctx.handle, key.handle, ctypes.c_void_p(d_big.data_ptr()),
                                  ctypes.c_void_p(d_out.data_ptr()), count, sh))

    for _ in range(warmup):
        step()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream.synchronize()
    a.record(stream)
    for _ in range(steps):
        step()
    b.record(stream)
    stream.synchronize()
    ms = a.elapsed_time(b)
    return {"workload": f"wwl24_t32_n2048_batch{count}", "params": params_config(p),
            "ciphertexts_per_step": count, "value": count * steps / (ms / 1e3), "unit": "bootstraps/s",
            "steps": steps, "ms_per_step": ms / steps, "launch_shape": tuning,
            "key_upload_s": min(uploads), "key_upload_s_all": uploads,
            "key_host_bytes": int(cprime.nbytes + s2.nbytes), "ginx_key_host_bytes": p.bsk_ntt_words * 8,
            "key_device_bytes": key.device_bytes}


def leg_lazy(dev, steps=3, warmup=1, count=1216, cpu_sample=16):
    """Lazy ("OURS") keys on the reference's default TORUS=32 set (n=680, N=2048, B=2^4,
    lApprox=4, s2 key with l=8 levels, KS 2^2 x 16): seeded synthetic half rows (uniform torus
    words, like a real key's coefficient-domain rows) and s2 key (uniform mod q), uploaded
    through yg_key_upload_lazy, then `count` bootstraps per step through
    yg_blind_rotate_extract (lazy_blind_rotate_kernel) and yg_keyswitch.  Reports the device
    key bytes beside the GINX key's, the upload time, the throughput, and the CPU restatement
    of blindRotateLazyPipeAltNtt on a `cpu_sample`-ciphertext sample with all host threads
    (also the bit-exact check of that sample)."""
    import torch

    from yatfhe_gb300 import _lib, api
    from yatfhe_gb300.params import WWL24_T32_N2048 as p

    rng = np.random.default_rng(0x5EED000A)
    row = (p.k + 1) * p.N
    cprime = rng.integers(-(1 << 31), 1 << 31, size=p.n * p.l_approx * row, dtype=np.int64)
    s2 = rng.integers(0, p.q_ntt, size=p.l * row, dtype=np.uint64)
    ksk = rng.integers(-(1 << 31), 1 << 31, size=p.ksk_words, dtype=np.int64).astype(np.int32)
    ctx = api.Context(p, dev)
    uploads = []
    for _ in range(3):  # the first call also pays one-time setup; the best of three is reported
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        key = api.BootstrapKey.from_lazy_words(ctx, cprime, s2)
        uploads.append(time.perf_counter() - t0)
        key.close()
    key = api.BootstrapKey.from_lazy_words(ctx, cprime, s2).set_ksk(ksk)
    lwe = synthetic_lwe(p, count, 0x5EED000B)
    lut = workload_lut(p)
    d_in = torch.from_numpy(lwe).to(f"cuda:{dev}")
    d_lut = torch.from_numpy(lut).to(f"cuda:{dev}")
    d_big = torch.empty((count, p.k * p.N + 1), dtype=torch.int32, device=f"cuda:{dev}")
    d_out = torch.empty_like(d_in)
    L = _lib.lib()
    stream = torch.cuda.Stream(device=dev)
    sh = ctypes.c_void_p(stream.cuda_stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * steps + 2)]

    def step(e0=None, e1=None):
        _lib.check(L.yg_blind_rotate_extract(ctx.handle, key.handle, ctypes.c_void_p(d_in.data_ptr()),
                                             ctypes.c_void_p(d_lut.data_ptr()), ctypes.c_void_p(d_big.data_ptr()),
                                             count, sh))
        if e1 is not None:
            e1.record(stream)
        _lib.check(L.yg_keyswitch(ctx.handle, key.handle, ctypes.c_void_p(d_big.data_ptr()),
                                  ctypes.c_void_p(d_out.data_ptr()), count, sh))

    for _ in range(warmup):
        step()
    stream.synchronize()
    ev[0].record(stream)
    marks = []
    for i in range(steps):
        b0 = ev[2 + 2 * i]
        b0.record(stream)
        step(e1=ev[3 + 2 * i])
        marks.append((b0, ev[3 + 2 * i]))
    ev[1].record(stream)
    stream.synchronize()
    ms = ev[0].elapsed_time(ev[1])
    br_ms = sum(x.elapsed_time(y) for x, y in marks) / steps
    value = count * steps / (ms / 1e3)
    # CPU baseline: the restatement of the lazy bootstrap, all host threads, on a sample
    from oracle.oracle import Restatement

    threads = os.cpu_count() or 1
    ora = Restatement(p)
    ora.set_lazy(cprime.reshape(p.n, p.l_approx, p.k + 1, p.N), s2.reshape(p.l, p.k + 1, p.N))
    ora.set_ksk(ksk)
    t0 = time.perf_counter()
    cpu_out = ora.pbs_lazy(lwe[:cpu_sample], lut, threads=threads)
    cpu_s = time.perf_counter() - t0
    bit_exact = bool(np.array_equal(cpu_out, d_out[:cpu_sample].cpu().numpy()))
    # butterflies of the kernel's transforms per bootstrap: per CMux step L batches of Ls + 3
    # forward transforms and one batch of 2 inverse ones, N/2 log2 N butterflies each
    logn = p.N.bit_length() - 1
    bfly = (p.n - 1) * (p.l_approx * (p.l + 3) + 2) * (p.N // 2) * logn
    return {"workload": f"lazy_t32_n2048_batch{count}", "params": dict(params_config(p), s2_levels=p.l),
            "ciphertexts_per_step": count, "value": value, "unit": "bootstraps/s", "steps": steps,
            "ms_per_step": ms / steps, "blind_rotate_ms_per_step": br_ms,
            "transform_butterflies_per_bootstrap": bfly,
            "butterflies_per_s": bfly * count / (br_ms / 1e3),
            "key_upload_s": min(uploads), "key_upload_s_all": uploads,
            "key_device_bytes": key.device_bytes, "ginx_key_device_bytes_same_set": p.n * p.l_approx * 4 * 3 * p.N * 4,
            "cpu_baseline": {"value": cpu_sample / cpu_s, "unit": "bootstraps/s", "cores": threads, "kind": "port",
                             "sample": f"{cpu_sample} of the step's ciphertexts, restatement of "
                                       "blindRotateLazyPipeAltNtt + extraction + key switching"},
            "sample_bit_exact": bit_exact}


def leg_group(dev, group=2, steps=3, warmup=1, count=9728, cpu_sample=32):
    """The group-g key family of blindRotateNtt (BootstrappingKey, param.group = g) on the
    TORUS=32 set (n=630, N=1024, B=2^7, l=lApprox=3): seeded synthetic TrgswDft words (uniform
    mod q), uploaded through yg_key_upload_group, then `count` bootstraps per step
    (functionalBootstrappingNtt: group_blind_rotate_kernel, then the key switch).  Reports the
    throughput, the device key bytes and the CPU restatement on a `cpu_sample`-ciphertext
    sample with all host threads (also the bit-exact check of that sample)."""
    import torch

    from yatfhe_gb300 import _lib, api
    from yatfhe_gb300.params import T32_N1024 as p

    rng = np.random.default_rng(0x5EED000C + group)
    keys = p.n if group == 1 else (p.n // group) << group
    words = rng.integers(0, p.q_ntt, size=keys * p.l * (p.k + 1) ** 2 * p.N, dtype=np.uint64)
    ksk = rng.integers(-(1 << 31), 1 << 31, size=p.ksk_words, dtype=np.int64).astype(np.int32)
    ctx = api.Context(p, dev)
    key = api.BootstrapKey.from_group_words(ctx, words, group).set_ksk(ksk)
    lwe = synthetic_lwe(p, count, 0x5EED0010 + group)
    lut = workload_lut(p)
    d_in = torch.from_numpy(lwe).to(f"cuda:{dev}")
    d_lut = torch.from_numpy(lut).to(f"cuda:{dev}")
    d_big = torch.empty((count, p.k * p.N + 1), dtype=torch.int32, device=f"cuda:{dev}")
    d_out = torch.empty_like(d_in)
    L = _lib.lib()
    stream = torch.cuda.Stream(device=dev)
    sh = ctypes.c_void_p(stream.cuda_stream)

    def step():
        _lib.check(L.yg_blind_rotate_extract(ctx.handle, key.handle, ctypes.c_void_p(d_in.data_ptr()),
                                             ctypes.c_void_p(d_lut.data_ptr()), ctypes.c_void_p(d_big.data_ptr()),
                                             count, sh))
        _lib.check(L.yg_keyswitch(ctx.handle, key.handle, ctypes.c_void_p(d_big.data_ptr()),
                                  ctypes.c_void_p(d_out.data_ptr()), count, sh))

    for _ in range(warmup):
        step()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream.synchronize()
    a.record(stream)
    for _ in range(steps):
        step()
    b.record(stream)
    stream.synchronize()
    ms = a.elapsed_time(b)
    from oracle.oracle import Restatement

    threads = os.cpu_count() or 1
    ora = Restatement(p)
    ora.set_group(words.reshape(keys, p.l, p.k + 1, p.k + 1, p.N), group)
    ora.set_ksk(ksk)
    t0 = time.perf_counter()
    cpu_out = ora.pbs_group(lwe[:cpu_sample], lut, threads=threads)
    cpu_s = time.perf_counter() - t0
    bit_exact = bool(np.array_equal(cpu_out, d_out[:cpu_sample].cpu().numpy()))
    return {"workload": f"group{group}_t32_n1024_batch{count}", "params": dict(params_config(p), group=group),
            "ciphertexts_per_step": count, "value": count * steps / (ms / 1e3), "unit": "bootstraps/s",
            "steps": steps, "ms_per_step": ms / steps, "key_device_bytes": key.device_bytes,
            "cpu_baseline": {"value": cpu_sample / cpu_s, "unit": "bootstraps/s", "cores": threads, "kind": "port",
                             "sample": f"{cpu_sample} of the step's ciphertexts, restatement of "
                                       "functionalBootstrappingNtt (blindRotateNtt on the group key)"},
            "sample_bit_exact": bit_exact}


def leg_keygen(dev, reps=3):
    """Key generation on the GPU for the TORUS=32 set (n=630, N=1024): seeded synthetic
    samples with the distributions of real ones (binary secrets, TUniform(2^8) / (2^18)
    noise, uniform masks), turned into a device key (BSK + KSK) by yg_keygen_from_samples;
    the best of `reps` wall times, the samples' host bytes."""
    import torch

    from yatfhe_gb300 import api
    from yatfhe_gb300.params import T32_N1024 as p

    rng = np.random.default_rng(0x5EED0007)
    k1, kN = p.k + 1, p.k * p.N
    smp = {"lwe_s": rng.integers(0, 2, p.n).astype(np.int32), "rlwe_s": rng.integers(0, 2, kN).astype(np.int32),
           "bsk_noise": rng.integers(-(1 << p.rlwe_noise_b), (1 << p.rlwe_noise_b) + 1,
                                     size=(p.n, p.l_approx, k1, p.N)).astype(np.int32),
           "bsk_mask": rng.integers(0, p.q_ntt, size=(p.n, p.l_approx, k1, p.k, p.N), dtype=np.uint64),
           "ksk_mask": rng.integers(-(1 << 31), 1 << 31, size=(kN, p.ks_level, p.n), dtype=np.int64).astype(np.int32),
           "ksk_noise": rng.integers(-(1 << p.lwe_noise_b), (1 << p.lwe_noise_b) + 1,
                                     size=(kN, p.ks_level)).astype(np.int32)}
    ctx = api.Context(p, dev)
    times = []
    for _ in range(reps):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        key = api.keygen_from_samples(ctx, smp)
        times.append(time.perf_counter() - t0)
        key.close()
    return {"params": params_config(p), "keygen_s": min(times), "keygen_s_all": times,
            "sample_host_bytes": int(sum(v.nbytes for v in smp.values()))}


def crt_ops_per_rotation(n, N):
    """Multiply-class 32-bit operations of one approximate-CRT blind rotation: per CMux step 16
    forward and 8 inverse transforms of (N/2) log2 N butterflies and 32 N key products, 3
    operations per modular product (one 24-bit channel, Shoup or Montgomery)."""
    lg = int(np.log2(N))
    return 3 * n * (24 * (N // 2) * lg + 32 * N)


def leg_crt(dev, count=2432, steps=3, warmup=1, cpu_sample=2):
    """The approximate-CRT blind rotation (blindRotateApproxCRTNtt with decompTrlweMcrt before
    and trlweMcrtToCrt + recompTrlweCrt after) at the reference's default size, n = 680,
    N = 2048 on the torus Q_CRT: seeded synthetic residue keys (uniform centred residues, the
    value range of real ones) and samples, `count` rotations per step timed with CUDA events on
    the launching stream; the CPU restatement on a `cpu_sample`-rotation sample (one thread)
    checks the sample bit for bit."""
    import torch

    from oracle.oracle import CRT_Q, crt_blind_rotate
    from yatfhe_gb300 import api

    n, N = 680, 2048
    rng = np.random.default_rng(0x5EED0015)
    bsk8 = np.empty((n, 4, 2, 2, 2, N), np.int8)
    for d, q in enumerate((251, 241, 239, 233)):
        bsk8[:, d] = rng.integers(-(q // 2), q // 2 + 1, size=bsk8[:, d].shape)
    t0 = time.perf_counter()
    key = api.CrtKey(bsk8, dev)
    upload_s = time.perf_counter() - t0
    cuda = f"cuda:{dev}"
    acc = rng.integers(-(CRT_Q // 2), CRT_Q // 2 + 1, size=(count, 2, N)).astype(np.int32)
    rot = rng.integers(0, 2 * N, size=(count, n)).astype(np.int32)
    d_acc, d_rot = torch.from_numpy(acc).to(cuda), torch.from_numpy(rot).to(cuda)
    d_out = torch.empty_like(d_acc)
    stream = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            key.blind_rotate(d_acc, d_rot, out=d_out, stream=stream)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        stream.synchronize()
        ev[0].record(stream)
        for _ in range(steps):
            key.blind_rotate(d_acc, d_rot, out=d_out, stream=stream)
        ev[1].record(stream)
        stream.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / steps
    value = count / (ms / 1e3)
    ops = crt_ops_per_rotation(n, N)
    peak = int32_peak(dev)
    out = d_out.cpu().numpy()
    t0 = time.perf_counter()
    same = all(np.array_equal(crt_blind_rotate(bsk8, acc[c], rot[c])[0], out[c]) for c in range(cpu_sample))
    cpu_s = time.perf_counter() - t0
    return {"workload": f"crt_n{n}_n{N}_batch{count}", "rotations_per_s": value, "ms_per_step": ms,
            "key_upload_s": upload_s, "key_device_bytes": key.device_bytes,
            "roofline": {"bound": "int32", "kernel": "crt_blind_rotate_kernel", "ops_per_rotation": ops,
                         "achieved": ops * value / 1e12, "peak": peak, "unit": "TOP/s",
                         "frac": ops * value / 1e12 / peak,
                         "peak_source": "measured: yg_probe_int32_rate (32-bit IMAD chains, all SMs)"},
            "cpu_baseline": {"value": cpu_sample / cpu_s, "unit": "rotations/s", "cores": 1, "kind": "port",
                             "sample": f"{cpu_sample} of the step's rotations, restatement of "
                                       "blindRotateApproxCRTNtt (one thread)"},
            "sample_bit_exact": bool(same)}


def leg_lone(dev, reps=20, warmup=3):
    """One ciphertext per yg_pbs call (TORUS=32 set) in every layout the parameters have: the
    latency of a lone bootstrap, CUDA events around `reps` back-to-back calls after `warmup`;
    every layout's output must equal the channel-row layout's."""
    import torch

    from yatfhe_gb300 import _lib, api
    from yatfhe_gb300.params import T32_N1024

    p = T32_N1024
    ctx = api.Context(p, dev)
    bsk, ksk = synthetic_keys(p, 0x5EED4000)
    key = api.BootstrapKey.from_ntt_words(ctx, bsk).set_ksk(ksk)
    d_lut = torch.from_numpy(workload_lut(p)).to(f"cuda:{dev}")
    d_in = torch.from_numpy(synthetic_lwe(p, 1, 0x5EED4001)).to(f"cuda:{dev}")
    d_out = torch.empty_like(d_in)
    s = torch.cuda.Stream(device=dev)
    L = _lib.lib()
    lat, outs = {}, {}
    for name, lay in (("channel", 0), ("channel_row", 1), ("row_cluster", 2), ("channel_cluster", 3)):
        if api.ctas_per_sm(ctx, 1, lay) < 1:
            continue
        api.set_launch(ctx, 1, 0, lay)

        def call():
            _lib.check(L.yg_pbs(ctx.handle, key.handle, ctypes.c_void_p(d_in.data_ptr()),
                                ctypes.c_void_p(d_out.data_ptr()), 1, ctypes.c_void_p(d_lut.data_ptr()),
                                ctypes.c_void_p(s.cuda_stream)))

        for _ in range(warmup):
            call()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        for _ in range(reps):
            call()
        b.record(s)
        s.synchronize()
        lat[name] = a.elapsed_time(b) / reps
        outs[name] = d_out.cpu().numpy().copy()
    key.close()
    ref = outs["channel_row"]
    return {"workload": "lone_t32_n1024", "latency_ms_by_layout": lat, "reps": reps,
            "identical_across_layouts": all((o == ref).all() for o in outs.values())}


def leg_encrypt(dev, count=1 << 20, steps=5, warmup=3, cpu_sample=20000):
    """symEncTlwe on the GPU for the TORUS=32 set (n=630): `count` messages per step encrypted
    by yg_encrypt_lwe (masks and TUniform(2^18) noise drawn by ChaCha20 in the kernel) and by
    yg_encrypt_lwe_from_samples (masks and noise read from HBM), timed with CUDA events on the
    launching stream (outputs of 2.6 GB, larger than L2); ciphertexts/s and the HBM view of
    the algorithmic bytes (drawn: 8 B message + 4 (n + 1) B ciphertext; from samples: + 4 n B
    mask + 4 B noise), and the CPU restatement (one thread, its sequential RNG) on a sample.
    Also yg_keygen's wall time (secrets, BSK and KSK from one seed, everything on the GPU) and
    yg_encrypt_rlwe_ntt on 16384 polynomials (N = 1024, masks and noise drawn on the GPU)."""
    import torch

    from yatfhe_gb300 import api
    from yatfhe_gb300.params import T32_N1024 as p

    ctx = api.Context(p, dev)
    times = []
    for _ in range(3):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        key = api.keygen(ctx, 0x5EED0011, p.lwe_noise_b, p.rlwe_noise_b)
        times.append(time.perf_counter() - t0)
        key.close()
    rng = np.random.default_rng(0x5EED0012)
    n = p.n
    cuda = f"cuda:{dev}"
    d_s = torch.from_numpy(rng.integers(0, 2, n).astype(np.int32)).to(cuda)
    d_mu = torch.from_numpy((rng.integers(0, 4, count) << 29).astype(np.int64)).to(cuda)
    d_mask = torch.from_numpy(rng.integers(-(1 << 31), 1 << 31, (count, n), dtype=np.int32)).to(cuda)
    d_noise = torch.from_numpy(rng.integers(-(1 << 18), (1 << 18) + 1, count).astype(np.int32)).to(cuda)
    d_out = torch.empty((count, n + 1), dtype=torch.int32, device=cuda)
    stream = torch.cuda.Stream(device=dev)
    hbm = measured_peaks().get("hbm_gbs", FALLBACK_HBM_GBS)

    def timed(fn, alg_bytes):
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                fn()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            stream.synchronize()
            ev[0].record(stream)
            for i in range(steps):
                fn(i)
            ev[1].record(stream)
            stream.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / steps
        gbs = alg_bytes / (ms / 1e3) / 1e9
        return {"ciphertexts_per_s": count / (ms / 1e3), "launch_ms": ms, "algorithmic_bytes": alg_bytes,
                "achieved_gbs": gbs, "hbm_frac": gbs / hbm}

    drawn = timed(lambda i=0: api.sym_enc_tlwe(ctx, d_s, d_mu, 7, i, p.lwe_noise_b, out=d_out, stream=stream),
                  count * (8 + 4 * (n + 1)))
    given = timed(lambda i=0: api.sym_enc_tlwe_from_samples(ctx, d_s, d_mu, d_mask, d_noise, out=d_out,
                                                            stream=stream),
                  count * (8 + 4 * (n + 1) + 4 * n + 4))
    del d_mask, d_noise
    rcount = 16384
    d_rs = torch.from_numpy(rng.integers(0, 2, p.k * p.N).astype(np.int32)).to(cuda)
    d_rmu = torch.from_numpy(rng.integers(-(1 << 31), 1 << 31, (rcount, p.N), dtype=np.int64)).to(cuda)
    d_rout = torch.empty((rcount, p.k + 1, p.N), dtype=torch.int64, device=cuda)
    rlwe = timed(lambda i=0: api.sym_enc_trlwe_ntt(ctx, d_rs, d_rmu, 9, i, p.rlwe_noise_b, out=d_rout, stream=stream),
                 rcount * p.N * (8 + 8 * (p.k + 1)))
    rlwe["samples_per_s"] = rlwe.pop("ciphertexts_per_s") * rcount / count
    rlwe["count"] = rcount
    from oracle.oracle import Restatement

    ora = Restatement(p)
    ora.keygen(0x5EED0013)
    mu = (rng.integers(0, 4, cpu_sample) << 29).astype(np.int64)
    t0 = time.perf_counter()
    ora.encrypt(mu)
    cpu_s = time.perf_counter() - t0
    rmu = rng.integers(-(1 << 31), 1 << 31, (200, p.N), dtype=np.int64)
    t0 = time.perf_counter()
    ora.encrypt_rlwe_ntt_samples(rmu)
    cpu_rlwe_s = time.perf_counter() - t0
    return {"params": params_config(p), "count": count, "keygen_seeded_s": min(times), "keygen_seeded_s_all": times,
            "encrypt_drawn": drawn, "encrypt_from_samples": given, "rlwe_encrypt_ntt_drawn": rlwe,
            "cpu_rlwe_encrypt_ntt": {"value": 200 / cpu_rlwe_s, "unit": "samples/s", "cores": 1, "kind": "port"},
            "hbm_peak_gbs": hbm,
            "cpu_baseline": {"value": cpu_sample / cpu_s, "unit": "ciphertexts/s", "cores": 1, "kind": "port",
                             "sample": f"{cpu_sample} encryptions by the restatement of symEncTlwe"}}


def leg_multi_tenant(dev, steps=2, warmup=1, total=32768):
    """32 tenants with their own keys: 24 on the TORUS=32 set, 8 on the TORUS=56 set;
    per-tenant ciphertext counts from Zipf(1.1) over the 32 tenants (32,768 draws).  Each
    parameter set is one multi-key plan (one blind-rotation + one key-switch launch over all
    its tenants, launch shape from the autotuner); both plans run concurrently on two
    streams inside ONE captured CUDA graph, and a step is one replay."""
    import torch

    from yatfhe_gb300 import api, autotune
    from yatfhe_gb300.params import T32_N1024, T56_N2048

    counts = zipf_counts(1.1, 32, total, 20260816)
    groups = []
    for p, tenants in ((T32_N1024, range(0, 24)), (T56_N2048, range(24, 32))):
        ctx = api.Context(p, dev)
        keys = []
        for t in tenants:
            bsk, ksk = synthetic_keys(p, 0x5EED1000 + t)
            keys.append(api.BootstrapKey.from_ntt_words(ctx, bsk).set_ksk(ksk))
        lut = torch.from_numpy(workload_lut(p)).to(f"cuda:{dev}")
        tuning = autotune.tune(ctx, keys[0], lut)
        key_ids = np.concatenate([np.full(counts[t], i, np.int32) for i, t in enumerate(tenants)])
        n_ct = len(key_ids)
        d_in = torch.from_numpy(synthetic_lwe(p, n_ct, 0x5EED1100 + p.torus_bits)).to(f"cuda:{dev}")
        d_out = torch.empty_like(d_in)
        plan = api.BatchPlan(ctx, keys, [lut], n_ct, key_ids=key_ids)
        groups.append({"ctx": ctx, "keys": keys, "lut": lut, "plan": plan, "d_in": d_in, "d_out": d_out,
                       "count": n_ct, "tenants": len(tenants), "tuning": tuning["choice"], "p": p})
    s_main, s_side = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)

    def launch_all():
        cur = torch.cuda.current_stream(dev)
        s_side.wait_stream(cur)
        with torch.cuda.stream(s_side):
            g = groups[1]
            g["plan"].run(g["d_in"], g["d_out"], stream=s_side)
        g = groups[0]
        g["plan"].run(g["d_in"], g["d_out"], stream=cur)
        cur.wait_stream(s_side)

    with torch.cuda.stream(s_main):
        launch_all()  # per-device kernel set-up happens outside the capture
    torch.cuda.synchronize(dev)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s_main):
        launch_all()
    for _ in range(warmup):
        graph.replay()
    torch.cuda.synchronize(dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(s_main):
        a.record(s_main)
        for _ in range(steps):
            graph.replay()
        b.record(s_main)
    torch.cuda.synchronize(dev)
    ms = a.elapsed_time(b) / steps
    # each parameter set alone (same plans, eager), to show what running them together buys
    alone = {}
    for g in groups:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(s_main):
            e0.record(s_main)
            g["plan"].run(g["d_in"], g["d_out"], stream=s_main)
            e1.record(s_main)
        torch.cuda.synchronize(dev)
        alone[f"t{g['p'].torus_bits}_ms"] = e0.elapsed_time(e1)
    out = {"workload": "mixed_t32x24_t56x8_zipf32768", "value": total / (ms / 1e3), "unit": "bootstraps/s",
           "steps": steps, "ms_per_step": ms, "graph": "one CUDA graph, 2 streams, 4 kernel launches per replay",
           "alone_ms": alone,
           "sets": [{"torus_bits": g["p"].torus_bits, "tenants": g["tenants"], "ciphertexts": g["count"],
                     "launch_shape": g["tuning"]} for g in groups],
           "tenant_counts": counts.tolist()}
    for g in groups:
        g["plan"].close()
        for k in g["keys"]:
            k.close()
    return out


def leg_serving(dev, requests=800, fractions=(0.5, 0.6, 0.7, 0.8, 0.9, 1.0), tenants=128, budget=4e9,
                max_count=256, max_batch=304, max_inflight=2, latency_batch_max=0):
    """128 tenants on the TORUS=32 set, requests of 1..256 ciphertexts (log-uniform) arriving
    as a Poisson process, tenants Zipf(1.1)-popular, BSK/KSK in an HBM LRU cache capped at
    4 GB with refills from pinned host memory.  First the peak rate is measured with the
    offered load far above capacity, then each fraction of it is offered; every output is
    compared with the same tenant's ciphertexts bootstrapped alone.  Batches of at most
    latency_batch_max ciphertexts (0: the library's default, two waves of six-CTA clusters)
    run in the channel-cluster latency layout."""
    import torch

    from yatfhe_gb300 import api, autotune, serving
    from yatfhe_gb300.params import T32_N1024

    p = T32_N1024
    ctx = api.Context(p, dev)
    lut_np = workload_lut(p)
    d_lut = torch.from_numpy(lut_np).to(f"cuda:{dev}")
    pool = torch.empty((tenants, max_count, p.n + 1), dtype=torch.int32).pin_memory()
    expect = torch.empty_like(pool).pin_memory()
    srv = None
    t_setup = time.perf_counter()
    for t in range(tenants):
        bsk, ksk = synthetic_keys(p, 0x5EED2000 + t)
        key = api.BootstrapKey.from_ntt_words(ctx, bsk).set_ksk(ksk)
        if srv is None:
            tuning = autotune.tune(ctx, key, d_lut, objective="latency")
            srv = serving.Server(ctx, key_budget_bytes=budget, max_batch=max_batch, max_inflight=max_inflight,
                                 max_tenants=tenants, latency_batch_max=latency_batch_max)
        lwe = synthetic_lwe(p, max_count, 0x5EED3000 + t)
        pool[t] = torch.from_numpy(lwe)
        d_in = pool[t].to(f"cuda:{dev}")
        expect[t] = api.functional_bootstrapping_mp_ntt(ctx, key, d_in, d_lut).cpu()
        srv.add_tenant(t, key, lut_np)
        key.close()  # the server keeps its own pinned-host image; HBM holds only the cache
    setup_s = time.perf_counter() - t_setup
    srv.start()
    slots = srv.counters()["key_slots"]
    peak = srv.run_trace(pool, expect, requests=max(requests, 1000), warmup=100, rate=1e6, seed=11,
                         max_count=max_count)
    peak_rps = peak["requests_per_s"]
    points = []
    mismatches = peak["mismatched_requests"]
    for i, f in enumerate(fractions):
        # SLO target 10 ms (this workload's p99 goal); the reference's 100 / 300 / 500 ms beside it
        r = srv.run_trace(pool, expect, requests=requests, warmup=100, rate=f * peak_rps, seed=100 + i,
                          max_count=max_count, slo_ms=10.0)
        mismatches += r["mismatched_requests"]
        points.append({"fraction_of_peak": f, "offered_rps": r["offered_rate"], "served": r["served"],
                       "requests_per_s": r["requests_per_s"], "bootstraps_per_s": r["ciphertexts_per_s"],
                       "p50_ms": r["sojourn"]["p50_ms"], "p99_ms": r["sojourn"]["p99_ms"],
                       "queue_p99_ms": r["queue"]["p99_ms"], "service_p50_ms": r["service"]["p50_ms"],
                       "hit_rate": r["hit_rate"], "key_misses": r["key_misses"], "batches": r["batches"],
                       "latency_layout_batches": r["latency_batches"],
                       "slo_ms": r["slo_ms"], "slo_violation_rate": r["slo_violation_rate"],
                       "slo_violation_rate_100": r["slo_violation_rate_100"],
                       "slo_violation_rate_300": r["slo_violation_rate_300"],
                       "slo_violation_rate_500": r["slo_violation_rate_500"],
                       "tenant_fairness_jain": r["tenant_fairness_jain"], "peak_queue_depth": r["peak_queue_depth"],
                       "load_concurrency_peak": r["load_concurrency_peak"],
                       "load_concurrency_mean": r["load_concurrency_mean"]})
    srv.close()
    at80 = min(points, key=lambda q: abs(q["fraction_of_peak"] - 0.8)) if points else None
    return {"workload": "serving_t32_128tenants_4GB", "tenants": tenants, "key_budget_bytes": int(budget),
            "key_slots": slots, "resident_fraction": slots / tenants, "max_batch": max_batch,
            "max_inflight": max_inflight, "request_sizes": f"floor(exp(U(0, ln {max_count + 1}))), 1..{max_count}",
            "launch_shape": tuning["choice"], "latency_batch_max": latency_batch_max,
            "peak": {"requests_per_s": peak_rps, "bootstraps_per_s": peak["ciphertexts_per_s"],
                     "p50_ms": peak["sojourn"]["p50_ms"], "p99_ms": peak["sojourn"]["p99_ms"],
                     "hit_rate": peak["hit_rate"]},
            "points": points, "at_80pct": at80, "mismatched_requests": mismatches,
            "bit_exact_vs_alone": mismatches == 0, "setup_s": setup_s}


def leg_serving_lazy(dev, requests=300, fractions=(0.5, 0.8), tenants=48, budget=4e9, max_count=64, max_batch=152,
                     max_inflight=2):
    """The serving loop with lazy ("OURS") keys on the reference's default TORUS=32 set (n=680,
    N=2048, lApprox=4, s2 key with 8 levels): 48 tenants with seeded synthetic half rows, s2
    keys and KSKs, a 4 GB HBM key budget, requests of 1..64 ciphertexts (log-uniform), Zipf(1.1)
    tenants, Poisson arrivals at fractions of the measured peak.  Reports how many tenants the
    budget holds against GINX keys of the same set, p50/p99, hit rate, and that every output
    equals the same ciphertexts bootstrapped alone."""
    import torch

    from yatfhe_gb300 import api, serving
    from yatfhe_gb300.params import WWL24_T32_N2048 as p

    ctx = api.Context(p, dev)
    lut_np = workload_lut(p)
    d_lut = torch.from_numpy(lut_np).to(f"cuda:{dev}")
    pool = torch.empty((tenants, max_count, p.n + 1), dtype=torch.int32).pin_memory()
    expect = torch.empty_like(pool).pin_memory()
    srv = serving.Server(ctx, key_budget_bytes=budget, max_batch=max_batch, max_inflight=max_inflight,
                         max_tenants=tenants)
    row = (p.k + 1) * p.N
    t_setup = time.perf_counter()
    key_bytes = 0
    for t in range(tenants):
        rng = np.random.default_rng(0x5EED4000 + t)
        cprime = rng.integers(-(1 << 31), 1 << 31, size=p.n * p.l_approx * row, dtype=np.int64)
        s2 = rng.integers(0, p.q_ntt, size=p.l * row, dtype=np.uint64)
        ksk = rng.integers(-(1 << 31), 1 << 31, size=p.ksk_words, dtype=np.int64).astype(np.int32)
        key = api.BootstrapKey.from_lazy_words(ctx, cprime, s2).set_ksk(ksk)
        key_bytes = key.device_bytes
        lwe = synthetic_lwe(p, max_count, 0x5EED5000 + t)
        pool[t] = torch.from_numpy(lwe)
        expect[t] = api.functional_bootstrapping_mp_ntt(ctx, key, pool[t].to(f"cuda:{dev}"), d_lut).cpu()
        srv.add_tenant(t, key, lut_np)
        key.close()
    setup_s = time.perf_counter() - t_setup
    srv.start()
    slots = srv.counters()["key_slots"]
    ginx_bytes = p.n * p.l_approx * 2 * 3 * 2 * p.N * 4 + p.ksk_words * 4  # device rows + KSK of a GINX key
    peak = srv.run_trace(pool, expect, requests=requests, warmup=20, rate=1e6, seed=21, max_count=max_count)
    points, mismatches = [], peak["mismatched_requests"]
    for i, f in enumerate(fractions):
        r = srv.run_trace(pool, expect, requests=requests, warmup=20, rate=f * peak["requests_per_s"], seed=200 + i,
                          max_count=max_count, slo_ms=100.0)
        mismatches += r["mismatched_requests"]
        points.append({"fraction_of_peak": f, "offered_rps": r["offered_rate"], "served": r["served"],
                       "bootstraps_per_s": r["ciphertexts_per_s"], "p50_ms": r["sojourn"]["p50_ms"],
                       "p99_ms": r["sojourn"]["p99_ms"], "hit_rate": r["hit_rate"], "key_misses": r["key_misses"],
                       "slo_violation_rate_100": r["slo_violation_rate_100"],
                       "tenant_fairness_jain": r["tenant_fairness_jain"]})
    srv.close()
    return {"workload": f"serving_lazy_t32_n2048_{tenants}tenants_4GB", "tenants": tenants,
            "key_budget_bytes": int(budget), "key_slots": slots, "lazy_key_device_bytes": key_bytes,
            "ginx_key_device_bytes_same_set": ginx_bytes, "ginx_slots_same_budget": int(budget // ginx_bytes),
            "request_sizes": f"floor(exp(U(0, ln {max_count + 1}))), 1..{max_count}",
            "peak": {"requests_per_s": peak["requests_per_s"], "bootstraps_per_s": peak["ciphertexts_per_s"],
                     "hit_rate": peak["hit_rate"]},
            "points": points, "mismatched_requests": mismatches, "bit_exact_vs_alone": mismatches == 0,
            "setup_s": setup_s}


# ------------------------------------------------------------------------------ reference arm

def reference_arm(args, p, config, threads):
    """The reference's CPU path (the oracle's plain-C restatement of
    functionalBootstrappingMPNtt, pinned bit-exact against the reference's own sources) on
    all host threads, a bounded sample of the workload per step."""
    bsk, ksk = synthetic_keys(p, 1234)
    lwe = synthetic_lwe(p, max(64, threads * 32), 1235)
    lut = workload_lut(p)
    sample = args.cpu_sample or max(16, threads * 32)  # a few seconds of CPU work per step
    for _ in range(args.warmup):
        run_cpu_baseline(p, bsk, ksk, lwe, lut, min(sample, threads), threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run_cpu_baseline(p, bsk, ksk, lwe, lut, sample, threads)
    wall = time.perf_counter() - t0
    v = args.steps * sample / wall
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "bootstraps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32/u64 torus",
        "data": "synthetic", "config": dict(config, cpu_sample_per_step=sample),
        "cpu_baseline": {"value": v, "unit": "bootstraps/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} ciphertexts per step of the same workload, plain-C restatement "
                                   f"of functionalBootstrappingMPNtt, {threads} threads"},
        "e2e": {"value": v, "unit": "bootstraps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def _safe(fn, dev, *a, **kw):
    """Runs one extra leg, recording its wall time and the clocks seen while it ran."""
    t0 = time.perf_counter()
    clocks = ClockSampler(dev)
    clocks.start()
    try:
        r = fn(dev, *a, **kw)
    except Exception as e:  # a failing extra leg is reported, the headline line still prints
        r = {"error": f"{type(e).__name__}: {e}", "trace": traceback.format_exc(limit=3)}
    r["clocks"] = clocks.stop()
    r["leg_seconds"] = time.perf_counter() - t0
    return r


def main():
    args = parse_args()
    rank, world, local = dist_env()
    from yatfhe_gb300.params import PARAM_SETS

    p = PARAM_SETS[args.params]
    count = args.count or (65536 if p.torus_bits == 32 else 16384)
    workload = f"{args.params}_batch{count}"
    config = {"workload": workload, "params": params_config(p), "ciphertexts_per_step": count, "per_rank": True}
    threads = cpu_threads()

    if args.impl == "reference":
        if rank == 0:
            reference_arm(args, p, config, threads)
        return

    import torch

    dev = local
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    if args.workload != "batch":
        if rank != 0:
            return
        if args.workload == "serving_lazy":
            r = leg_serving_lazy(dev)
            line = {"metric": "serving with lazy keys: tenants resident in 4 GB", "value": r["key_slots"],
                    "unit": "tenants", "n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                    "dtype": "int32 torus / u64 mod q", "data": "synthetic",
                    "config": {"workload": r["workload"]}, "result": r}
            print(json.dumps(line))
            return
        if args.workload == "crt":
            r = leg_crt(dev)
            line = {"metric": "approximate-CRT blind rotations per second", "value": r["rotations_per_s"],
                    "unit": "rotations/s", "n_gpus": 1, "higher_is_better": True, "scaling": "weak",
                    "vs_baseline": None, "dtype": "int8 residues / u32 mod 2^24-2^14+1", "data": "synthetic",
                    "config": {"workload": r["workload"]}, "result": r}
            print(json.dumps(line))
            return
        if args.workload == "lone":
            r = leg_lone(dev)
            line = {"metric": "lone-ciphertext bootstrap latency", "value": min(r["latency_ms_by_layout"].values()),
                    "unit": "ms", "n_gpus": 1, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                    "dtype": "int32 torus / u32 RNS", "data": "synthetic",
                    "config": {"workload": r["workload"]}, "result": r}
            print(json.dumps(line))
            return
        if args.workload == "encrypt":
            r = leg_encrypt(dev)
            line = {"metric": "LWE encryptions per second", "value": r["encrypt_drawn"]["ciphertexts_per_s"],
                    "unit": "ciphertexts/s", "n_gpus": 1, "higher_is_better": True, "scaling": "weak",
                    "vs_baseline": None, "dtype": "u32", "data": "synthetic",
                    "config": {"workload": "encrypt_t32_n630_batch1048576"}, "result": r}
            print(json.dumps(line))
            return
        if args.workload == "multi_tenant":
            r = leg_multi_tenant(dev, steps=args.steps, warmup=args.warmup)
            line = {"metric": METRIC, "value": r["value"], "unit": "bootstraps/s", "n_gpus": 1,
                    "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                    "dtype": "int32 torus / u32 RNS", "data": "synthetic",
                    "config": {"workload": r["workload"]}, "result": r}
        else:
            fr = tuple(float(x) for x in args.serving_fractions.split(","))
            r = leg_serving(dev, requests=args.serving_requests, fractions=fr, max_batch=args.serving_max_batch,
                            max_inflight=args.serving_inflight)
            a80 = r["at_80pct"] or {}
            line = {"metric": "serving p99 sojourn at 80% of peak", "value": a80.get("p99_ms"), "unit": "ms",
                    "n_gpus": 1, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                    "dtype": "int32 torus / u32 RNS", "data": "synthetic",
                    "config": {"workload": r["workload"]}, "result": r}
        print(json.dumps(line))
        return

    run = BatchRun(p, count, dev, seed=1234 + rank, per_cta=args.per_cta, ctas_per_sm=args.ctas_per_sm,
                   retune=args.retune, layout=args.layout)
    t = run.timed(args.steps, args.warmup, barrier=barrier, clocks=ClockSampler(dev))
    total_ms = t["total_ms"]
    if world > 1:
        import torch.distributed as dist

        tt = torch.tensor([total_ms], device=f"cuda:{dev}")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total_ms = float(tt.item())
    value = world * count * args.steps / (total_ms / 1e3)

    # end to end through the host-buffer entry point, pinned buffers
    L = run.L
    from yatfhe_gb300 import _lib, api

    h_in = torch.from_numpy(run.lwe).pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    h_lut = torch.from_numpy(run.lut).pin_memory()

    def e2e_step():
        _lib.check(L.yg_pbs_host(run.ctx.handle, run.key.handle, ctypes.c_void_p(h_in.data_ptr()),
                                 ctypes.c_void_p(h_out.data_ptr()), count, ctypes.c_void_p(h_lut.data_ptr()), run.sh))

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_value = world * count * args.steps / e2e_s
    if not torch.equal(h_out, run.d_out.cpu()):
        raise SystemExit("host-buffer and device-buffer entry points disagree")

    if rank != 0:
        return

    roofline = run.roofline(t["br_ms"], int32_peak(dev), workload)
    roofline["keyswitch_ms"] = statistics.mean(t["ks_ms"])

    extras = {}
    if not args.no_extras:
        d_in, d_out, d_lut, sh = run.d_in, run.d_out, run.d_lut, run.sh
        # plain per-call form: one ciphertext per launch
        one_in, one_out = d_in[:1], d_out[:1]

        def pbs(src, dst, n):
            _lib.check(L.yg_pbs(run.ctx.handle, run.key.handle, ctypes.c_void_p(src.data_ptr()),
                                ctypes.c_void_p(dst.data_ptr()), n, ctypes.c_void_p(d_lut.data_ptr()), sh))

        for _ in range(3):
            pbs(one_in, one_out, 1)
        run.stream.synchronize()
        reps = 20
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(run.stream)
        for _ in range(reps):
            pbs(one_in, one_out, 1)
        b.record(run.stream)
        run.stream.synchronize()
        extras["plain_per_call_bps"] = reps / (a.elapsed_time(b) / 1e3)
        extras["plain_per_call_latency_ms"] = a.elapsed_time(b) / reps
        sweep = {}
        for bs in (1, 64, 1024):
            if bs > count:
                continue
            a.record(run.stream)
            for _ in range(2):
                pbs(d_in, d_out, bs)
            b.record(run.stream)
            run.stream.synchronize()
            sweep[str(bs)] = 2 * bs / (a.elapsed_time(b) / 1e3)
        sweep[str(count)] = value / world
        extras["batch_sweep_bps"] = sweep
        extras["batched_over_plain"] = value / world / extras["plain_per_call_bps"]
        # one ciphertext per call in each layout that exists for these parameters (one
        # ciphertext per CTA), then the tuned shape back
        lone = {}
        for name, lay in (("channel", 0), ("channel_row", 1), ("row_cluster", 2), ("channel_cluster", 3)):
            if api.ctas_per_sm(run.ctx, 1, lay) < 1:
                continue
            api.set_launch(run.ctx, 1, 0, lay)
            for _ in range(3):
                pbs(one_in, one_out, 1)
            a.record(run.stream)
            for _ in range(10):
                pbs(one_in, one_out, 1)
            b.record(run.stream)
            run.stream.synchronize()
            lone[name] = a.elapsed_time(b) / 10
        c = run.tuning["choice"]
        api.set_launch(run.ctx, c["per_cta"], c["ctas_per_sm"], c.get("layout", 0))
        extras["lone_latency_ms_by_layout"] = lone

    # CPU baseline on a bounded sample (oracle on the host cores), also the bit-exact check;
    # the step's outputs are recomputed first (the sweep above overwrote part of them)
    run.step()
    run.stream.synchronize()
    sample = args.cpu_sample or max(16, threads * 48)  # about 10 s of CPU work
    cpu_out, cpu_bps, cpu_s, cpu_lat = run_cpu_baseline(p, run.bsk, run.ksk, run.lwe, run.lut, sample, threads,
                                                        latency=True)
    bit_exact = bool(np.array_equal(cpu_out, run.d_out[:sample].cpu().numpy()))

    if not args.no_extras:
        extras["workloads"] = {
            "t56_n2048_batch16384": _safe(leg_t56, dev),
            "wwl24_t32_n2048_batch16384": _safe(leg_wwl24, dev),
            "keygen_t32_n1024": _safe(leg_keygen, dev),
            "encrypt_t32_n630_batch1048576": _safe(leg_encrypt, dev),
            "crt_n680_n2048_batch2432": _safe(leg_crt, dev),
            "lazy_t32_n2048_batch1216": _safe(leg_lazy, dev),
            "group2_t32_n1024_batch9728": _safe(leg_group, dev, 2),
            "group3_t32_n1024_batch9728": _safe(leg_group, dev, 3),
            "mixed_t32x24_t56x8_zipf32768": _safe(leg_multi_tenant, dev),
            "serving_t32_128tenants_4GB": _safe(
                leg_serving, dev, requests=args.serving_requests,
                fractions=tuple(float(x) for x in args.serving_fractions.split(",")),
                max_batch=args.serving_max_batch, max_inflight=args.serving_inflight),
            "serving_lazy_t32_n2048_48tenants_4GB": _safe(leg_serving_lazy, dev),
        }

    line = {
        "metric": METRIC, "value": value, "unit": "bootstraps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32 torus / u32 RNS", "data": "synthetic",
        "config": dict(config, l2="inputs larger than L2 (%.0f MB in + %.0f MB extract per step > %d MB)"
                       % (count * (p.n + 1) * 4 / 1e6, count * (p.N + 1) * 4 / 1e6, L2_BYTES // 2**20),
                       parallelism=f"replicas x{world}"),
        "clocks": t["clocks"],
        "e2e": {"value": e2e_value, "unit": "bootstraps/s", "h2d_bytes_per_step": count * (p.n + 1) * 4 + p.N * 8,
                "d2h_bytes_per_step": count * (p.n + 1) * 4, "entry_point": "yg_pbs_host"},
        "gpu_launches": 2 * args.steps,
        "roofline": roofline,
        "cpu_baseline": {"value": cpu_bps, "unit": "bootstraps/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} of the step's ciphertexts, plain-C restatement of "
                                   f"functionalBootstrappingMPNtt on {threads} threads ({cpu_s:.1f} s)",
                         "latency_ms_one_thread": cpu_lat},
        "bit_exact_vs_oracle_sample": bit_exact,
        "key_upload_s": run.key_upload_s,
        "launch_shape": run.tuning,
        "key_device_bytes": run.key.device_bytes,
    }
    line.update(extras)
    print(json.dumps(line))


if __name__ == "__main__":
    main()

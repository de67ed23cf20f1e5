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
which also checks the sampled GPU outputs bit for bit.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--params t32_n1024|t56_n2048]
                  [--count C] [--impl ours|reference]
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "bootstraps/s"
L2_BYTES = 129 * 2**20


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--params", default="t32_n1024")
    ap.add_argument("--count", type=int, default=0, help="ciphertexts per step (default 65536 / 16384)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extras", action="store_true", help="skip the per-call / batch-size sweep legs")
    ap.add_argument("--cpu-sample", type=int, default=0, help="ciphertexts in the CPU baseline sample")
    ap.add_argument("--per-cta", type=int, default=0, help="fix ciphertexts per CTA (skips the autotuner)")
    ap.add_argument("--ctas-per-sm", type=int, default=0, help="with --per-cta: persistent CTAs per SM (0 = off)")
    ap.add_argument("--retune", action="store_true", help="re-measure launch shapes instead of the cached choice")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def synthetic(p, count, seed):
    """Seeded synthetic inputs with the shapes of a real key set: NTT-domain BSK words are
    uniform mod q (as a real key's are: its masks are sampled uniformly in that domain), KSK
    and ciphertext words uniform mod 2^32 (as real masks are)."""
    rng = np.random.default_rng(seed)
    bsk = rng.integers(0, p.q_ntt, size=p.bsk_ntt_words, dtype=np.uint64)
    ksk = rng.integers(-(1 << 31), 1 << 31, size=p.ksk_words, dtype=np.int64).astype(np.int32)
    lwe = rng.integers(-(1 << 31), 1 << 31, size=(count, p.n + 1), dtype=np.int64).astype(np.int32)
    from yatfhe_gb300 import lut as lutmod

    lut = lutmod.sign_lut(p.N, p.torus_bits)
    return bsk, ksk, lwe, lut


def ops_per_bootstrap(p):
    """Multiply-class 32-bit operations per bootstrap: 9 per mod-q multiplication (3 RNS
    channels x 3 for a Shoup word multiply) over the blind rotation's modmul count
    M = n [2l (N/2) log2 N + 4 l N + 2 (N/2) log2 N], plus the key switch's k N t (n+1) MACs."""
    logN = int(np.log2(p.N))
    L = p.l_approx
    M = p.n * (2 * L * (p.N // 2) * logN + 4 * L * p.N + 2 * (p.N // 2) * logN)
    ks = p.k * p.N * p.ks_level * (p.n + 1)
    return 9 * M, ks


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
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


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


def run_cpu_baseline(p, bsk, ksk, lwe, lut, sample, threads):
    """The CPU oracle (plain-C restatement of the reference path) on `sample` ciphertexts."""
    from oracle.oracle import Restatement

    ora = Restatement(p)
    ora.set_bsk_ntt(bsk)
    ora.set_ksk(ksk)
    t0 = time.perf_counter()
    out = ora.pbs(lwe[:sample], lut, threads=threads)
    dt = time.perf_counter() - t0
    return out, sample / dt, dt


def main():
    args = parse_args()
    rank, world, local = dist_env()
    from yatfhe_gb300.params import PARAM_SETS

    p = PARAM_SETS[args.params]
    count = args.count or (65536 if p.torus_bits == 32 else 16384)
    workload = f"{args.params}_batch{count}"
    config = {"workload": workload, "params": {"n": p.n, "N": p.N, "k": p.k, "B": 1 << p.radix_bits,
                                                 "l": p.l_approx, "ks_base": 1 << p.ks_radix_bits,
                                                 "ks_t": p.ks_level, "torus_bits": p.torus_bits},
              "ciphertexts_per_step": count, "per_rank": True}
    threads = cpu_threads()

    if args.impl == "reference":
        if rank != 0:
            return
        bsk, ksk, lwe, lut = synthetic(p, max(64, threads * 4), 1234)
        sample = args.cpu_sample or max(16, threads * 2)
        for _ in range(args.warmup):
            run_cpu_baseline(p, bsk, ksk, lwe, lut, min(sample, threads), threads)
        rates = []
        t0 = time.perf_counter()
        for _ in range(args.steps):
            _, r, _ = run_cpu_baseline(p, bsk, ksk, lwe, lut, sample, threads)
            rates.append(r)
        wall = time.perf_counter() - t0
        v = args.steps * sample / wall
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": v, "unit": "bootstraps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32/u64 torus",
            "data": "synthetic", "config": dict(config, cpu_sample_per_step=sample),
            "cpu_baseline": {"value": v, "unit": "bootstraps/s", "cores": threads, "kind": "port",
                             "sample": f"{sample} ciphertexts per step of the same workload, plain-C restatement "
                                       f"of functionalBootstrappingMPNtt, {threads} threads"},
            "e2e": {"value": v, "unit": "bootstraps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }))
        return

    import torch

    from yatfhe_gb300 import _lib, api

    dev = local
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    L = _lib.lib()

    bsk, ksk, lwe, lut = synthetic(p, count, 1234 + rank)
    ctx = api.Context(p, dev)
    t_key = time.perf_counter()
    key = api.BootstrapKey.from_ntt_words(ctx, bsk).set_ksk(ksk)
    key_upload_s = time.perf_counter() - t_key

    stream = torch.cuda.Stream()
    sh = ctypes.c_void_p(stream.cuda_stream)
    d_in = torch.from_numpy(lwe).to(f"cuda:{dev}")
    d_lut = torch.from_numpy(lut).to(f"cuda:{dev}")
    if args.per_cta:
        api.set_launch(ctx, args.per_cta, args.ctas_per_sm)
        tuning = {"choice": {"per_cta": args.per_cta, "ctas_per_sm": args.ctas_per_sm}, "fixed": True}
    else:
        from yatfhe_gb300 import autotune

        tuning = autotune.tune(ctx, key, d_lut, use_cache=not args.retune)
    d_big = torch.empty((count, p.k * p.N + 1), dtype=torch.int32, device=f"cuda:{dev}")
    d_out = torch.empty_like(d_in)
    torch.cuda.synchronize()

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        _lib.check(L.yg_blind_rotate_extract(ctx.handle, key.handle, ctypes.c_void_p(d_in.data_ptr()),
                                             ctypes.c_void_p(d_lut.data_ptr()), ctypes.c_void_p(d_big.data_ptr()),
                                             count, sh))
        if ev:
            ev[1].record(stream)
        _lib.check(L.yg_keyswitch(ctx.handle, key.handle, ctypes.c_void_p(d_big.data_ptr()),
                                  ctypes.c_void_p(d_out.data_ptr()), count, sh))
        if ev:
            ev[2].record(stream)

    for _ in range(args.warmup):
        step()
    stream.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(dev)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    clocks.start()
    start.record(stream)
    for k in range(args.steps):
        step(evs[k])
    end.record(stream)
    stream.synchronize()
    barrier()
    clock_info = clocks.stop()
    total_ms = start.elapsed_time(end)
    br_ms = [e[0].elapsed_time(e[1]) for e in evs]
    ks_ms = [e[1].elapsed_time(e[2]) for e in evs]
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([total_ms], device=f"cuda:{dev}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * count * args.steps / (total_ms / 1e3)

    # end to end through the host-buffer entry point, pinned buffers
    h_in = torch.from_numpy(lwe).pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    h_lut = torch.from_numpy(lut).pin_memory()

    def e2e_step():
        _lib.check(L.yg_pbs_host(ctx.handle, key.handle, ctypes.c_void_p(h_in.data_ptr()),
                                 ctypes.c_void_p(h_out.data_ptr()), count, ctypes.c_void_p(h_lut.data_ptr()), sh))

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_value = world * count * args.steps / e2e_s
    if not torch.equal(h_out, d_out.cpu()):
        raise SystemExit("host-buffer and device-buffer entry points disagree")

    if rank != 0:
        return

    # roofline of the dominant kernel (blind rotation + extract), against the measured
    # 32-bit multiply-add rate of this GPU
    rate = ctypes.c_double()
    _lib.check(L.yg_probe_int32_rate(dev, ctypes.byref(rate)))
    br_ops, ks_ops = ops_per_bootstrap(p)
    br_avg_s = statistics.mean(br_ms) / 1e3
    achieved = br_ops * count / br_avg_s / 1e12
    peak = rate.value / 1e12
    bsk_alg = p.n * p.l_approx * (p.k + 1) ** 2 * p.N * 8
    io_alg = count * ((p.n + 1) + (p.k * p.N + 1)) * 4
    hbm = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"] if (
        ROOT / "MEASURED_PEAKS.json").exists() else 6800.0
    hbm_achieved = (bsk_alg + io_alg) / br_avg_s / 1e9
    roofline = {
        "bound": "int32", "kernel": "blind_rotate_kernel", "achieved": achieved, "peak": peak, "unit": "TOP/s",
        "frac": achieved / peak, "peak_source": "measured: yg_probe_int32_rate (32-bit IMAD chains, all SMs)",
        "ops_per_bootstrap": br_ops, "launch_ms": statistics.mean(br_ms),
        "traffic": traffic_from_profiles("blind_rotate_kernel", workload),
        "hbm_view": {"algorithmic_bytes_per_launch": bsk_alg + io_alg, "achieved_gbs": hbm_achieved,
                     "peak_gbs": hbm, "frac": hbm_achieved / hbm, "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "keyswitch_ms": statistics.mean(ks_ms),
    }

    extras = {}
    if not args.no_extras:
        # plain per-call form: one ciphertext per launch
        one_in, one_out = d_in[:1], d_out[:1]
        for _ in range(3):
            _lib.check(L.yg_pbs(ctx.handle, key.handle, ctypes.c_void_p(one_in.data_ptr()),
                                ctypes.c_void_p(one_out.data_ptr()), 1, ctypes.c_void_p(d_lut.data_ptr()), sh))
        stream.synchronize()
        reps = 20
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            _lib.check(L.yg_pbs(ctx.handle, key.handle, ctypes.c_void_p(one_in.data_ptr()),
                                ctypes.c_void_p(one_out.data_ptr()), 1, ctypes.c_void_p(d_lut.data_ptr()), sh))
        b.record(stream)
        stream.synchronize()
        extras["plain_per_call_bps"] = reps / (a.elapsed_time(b) / 1e3)
        sweep = {}
        for bs in (1, 64, 1024):
            if bs > count:
                continue
            a.record(stream)
            for _ in range(2):
                _lib.check(L.yg_pbs(ctx.handle, key.handle, ctypes.c_void_p(d_in.data_ptr()),
                                    ctypes.c_void_p(d_out.data_ptr()), bs, ctypes.c_void_p(d_lut.data_ptr()), sh))
            b.record(stream)
            stream.synchronize()
            sweep[str(bs)] = 2 * bs / (a.elapsed_time(b) / 1e3)
        sweep[str(count)] = value / world
        extras["batch_sweep_bps"] = sweep
        extras["batched_over_plain"] = value / world / extras["plain_per_call_bps"]

    # CPU baseline on a bounded sample (oracle on the host cores), also the bit-exact check
    sample = args.cpu_sample or max(16, threads * 4)
    cpu_out, cpu_bps, cpu_s = run_cpu_baseline(p, bsk, ksk, lwe, lut, sample, threads)
    bit_exact = bool(np.array_equal(cpu_out, d_out[:sample].cpu().numpy()))

    line = {
        "metric": METRIC, "value": value, "unit": "bootstraps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32 torus / u32 RNS", "data": "synthetic",
        "config": dict(config, l2="inputs larger than L2 (%.0f MB in + %.0f MB extract per step > %d MB)"
                       % (count * (p.n + 1) * 4 / 1e6, count * (p.N + 1) * 4 / 1e6, L2_BYTES // 2**20),
                       parallelism=f"replicas x{world}"),
        "clocks": clock_info,
        "e2e": {"value": e2e_value, "unit": "bootstraps/s", "h2d_bytes_per_step": count * (p.n + 1) * 4 + p.N * 8,
                "d2h_bytes_per_step": count * (p.n + 1) * 4, "entry_point": "yg_pbs_host"},
        "gpu_launches": 2 * args.steps,
        "roofline": roofline,
        "cpu_baseline": {"value": cpu_bps, "unit": "bootstraps/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} of the step's ciphertexts, plain-C restatement of "
                                   f"functionalBootstrappingMPNtt on {threads} threads ({cpu_s:.1f} s)"},
        "bit_exact_vs_oracle_sample": bit_exact,
        "key_upload_s": key_upload_s,
        "launch_shape": tuning,
        "key_device_bytes": key.device_bytes,
    }
    line.update(extras)
    print(json.dumps(line))


if __name__ == "__main__":
    main()

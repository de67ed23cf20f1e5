"""Launch-shape autotuner for the blind-rotation kernel.

The knobs (yg_ctx_set_launch / yg_plan_set_launch):
  per_cta      ciphertexts per CTA run in lockstep (1, 2, 4 at N = 1024; 1, 2 at N = 2048):
               more share instruction-cache lines and key lines in L1, fewer keep more
               independent CTAs per SM;
  ctas_per_sm  0 = one CTA per group of per_cta ciphertexts (the hardware scheduler fills
               the SMs), c > 0 = a persistent grid of c CTAs per SM looping over the batch.
Each candidate that fits an SM is timed with CUDA events on a sample batch; the fastest is
applied to the context and cached in yatfhe_gb300/_build/autotune.json per (GPU,
parameter set), so later processes reuse it without measuring.
"""
from __future__ import annotations

import json
import os
from dataclasses import asdict
from pathlib import Path

import numpy as np

from . import api

CACHE = Path(__file__).resolve().parent / "_build" / "autotune.json"


def _key(ctx) -> str:
    import torch

    name = torch.cuda.get_device_name(ctx.device)
    return f"{name}|" + ",".join(f"{k}={v}" for k, v in sorted(asdict(ctx.params).items()))


def _load() -> dict:
    try:
        return json.loads(CACHE.read_text())
    except (OSError, ValueError):
        return {}


def _store(table: dict) -> None:
    CACHE.parent.mkdir(exist_ok=True)
    tmp = CACHE.with_suffix(f".tmp{os.getpid()}")
    tmp.write_text(json.dumps(table, indent=1, sort_keys=True))
    os.replace(tmp, CACHE)


def candidates(ctx) -> list[tuple[int, int]]:
    out = []
    for per_cta in (1, 2, 4):
        try:
            fit = api.ctas_per_sm(ctx, per_cta)
        except ValueError:
            continue
        if fit < 1:
            continue
        out.append((per_cta, 0))
        out.append((per_cta, fit))
    return out


def measure(ctx, key, lut, count: int, per_cta: int, ctas_per_sm: int, reps: int = 2, seed: int = 0) -> float:
    """Bootstraps per second of one launch shape on `count` random ciphertexts."""
    import torch

    sms = torch.cuda.get_device_properties(ctx.device).multi_processor_count
    rng = np.random.default_rng(seed)
    lwe = rng.integers(-(1 << 31), 1 << 31, size=(count, ctx.params.n + 1), dtype=np.int64).astype(np.int32)
    d_in = torch.from_numpy(lwe).to(f"cuda:{ctx.device}")
    d_out = torch.empty_like(d_in)
    plan = api.BatchPlan(ctx, [key], [lut], count, per_cta=per_cta, grid=ctas_per_sm * sms)
    s = torch.cuda.Stream(device=ctx.device)
    with torch.cuda.stream(s):
        plan.run(d_in, d_out, stream=s)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        for _ in range(reps):
            plan.run(d_in, d_out, stream=s)
        b.record(s)
    s.synchronize()
    plan.close()
    return reps * count / (a.elapsed_time(b) / 1e3)


def tune(ctx, key, lut, count: int | None = None, use_cache: bool = True, verbose: bool = False) -> dict:
    """Picks, applies and caches the fastest launch shape; returns {choice, results, cached}."""
    import torch

    k = _key(ctx)
    table = _load() if use_cache else {}
    if k in table:
        c = table[k]
        api.set_launch(ctx, c["per_cta"], c["ctas_per_sm"])
        return {"choice": c, "cached": True}
    sms = torch.cuda.get_device_properties(ctx.device).multi_processor_count
    if count is None:
        count = sms * 16  # several waves for every candidate
    results = []
    for per_cta, cps in candidates(ctx):
        bps = measure(ctx, key, lut, count, per_cta, cps)
        results.append({"per_cta": per_cta, "ctas_per_sm": cps, "bootstraps_per_s": bps})
        if verbose:
            print(f"autotune {per_cta}/CTA, {cps or 'all'} CTAs/SM: {bps:.0f} bootstraps/s")
    best = max(results, key=lambda r: r["bootstraps_per_s"])
    table = _load()
    table[k] = {**best, "sample": count}
    _store(table)
    api.set_launch(ctx, best["per_cta"], best["ctas_per_sm"])
    return {"choice": table[k], "results": results, "cached": False}

"""Launch-shape autotuner for the blind-rotation kernel.

The knobs (yg_ctx_set_launch / yg_plan_set_launch):
  layout       work split of one ciphertext: a thread team per RNS channel (LAYOUT_CHANNEL),
               per channel and accumulator row (LAYOUT_CHANNEL_ROW: twice the threads,
               about half the latency per ciphertext), a two-CTA cluster per ciphertext
               with a team per channel and digit level in each (LAYOUT_ROW_CLUSTER, T32 at
               N = 1024: the levels' transforms side by side), or a six-CTA cluster with a
               CTA per accumulator row and channel and a warp per digit level
               (LAYOUT_CHANNEL_CLUSTER, same limits: the shortest latency);
  per_cta      ciphertexts per CTA, sharing its L1 (1, 2, 4 at N = 1024; 1, 2 at N = 2048):
               more share instruction-cache lines and key lines in L1, fewer keep more
               independent CTAs per SM;
  ctas_per_sm  0 = one CTA per group of per_cta ciphertexts (the hardware scheduler fills
               the SMs), c > 0 = a persistent grid of c CTAs per SM looping over the batch.
Each candidate that fits an SM is timed with CUDA events on a sample batch (throughput)
and on one ciphertext alone (latency); the best for the objective -- the most bootstraps
per second, or for serving the lowest lone-ciphertext latency within 15 % of that -- is
applied to the context and cached in yatfhe_gb300/_build/autotune.json per (GPU,
parameter set, objective), so later processes reuse it without measuring.
"""
from __future__ import annotations

import json
import os
from dataclasses import asdict
from pathlib import Path

import numpy as np

from . import _lib, api

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


def candidates(ctx) -> list[tuple[int, int, int]]:
    """(layout, per_cta, ctas_per_sm) shapes that fit an SM."""
    out = []
    clusters = (_lib.LAYOUT_ROW_CLUSTER, _lib.LAYOUT_CHANNEL_CLUSTER)
    for layout in (_lib.LAYOUT_CHANNEL, _lib.LAYOUT_CHANNEL_ROW) + clusters:
        for per_cta in (1, 2, 4):
            try:
                fit = api.ctas_per_sm(ctx, per_cta, layout)
            except ValueError:
                continue
            if fit < 1:
                continue
            out.append((layout, per_cta, 0))
            if layout not in clusters:  # a fixed cluster per ciphertext, never persistent
                out.append((layout, per_cta, fit))
    return out


def measure(ctx, key, lut, count: int, per_cta: int, ctas_per_sm: int, reps: int = 2, seed: int = 0,
            layout: int = 0) -> tuple[float, float]:
    """(bootstraps per second on `count` random ciphertexts, milliseconds for one ciphertext
    alone) of one launch shape."""
    import torch

    sms = torch.cuda.get_device_properties(ctx.device).multi_processor_count
    rng = np.random.default_rng(seed)
    lwe = rng.integers(-(1 << 31), 1 << 31, size=(count, ctx.params.n + 1), dtype=np.int64).astype(np.int32)
    d_in = torch.from_numpy(lwe).to(f"cuda:{ctx.device}")
    d_out = torch.empty_like(d_in)
    plan = api.BatchPlan(ctx, [key], [lut], count, per_cta=per_cta, grid=ctas_per_sm * sms, layout=layout)
    one = api.BatchPlan(ctx, [key], [lut], 1, per_cta=per_cta, layout=layout)
    s = torch.cuda.Stream(device=ctx.device)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    with torch.cuda.stream(s):
        plan.run(d_in, d_out, stream=s)
        ev[0].record(s)
        for _ in range(reps):
            plan.run(d_in, d_out, stream=s)
        ev[1].record(s)
        one.run(d_in[:1], d_out[:1], stream=s)
        ev[2].record(s)
        for _ in range(reps):
            one.run(d_in[:1], d_out[:1], stream=s)
        ev[3].record(s)
    s.synchronize()
    plan.close()
    one.close()
    return reps * count / (ev[0].elapsed_time(ev[1]) / 1e3), ev[2].elapsed_time(ev[3]) / reps


OBJECTIVES = ("throughput", "latency")


LATENCY_WINDOW = 0.85  # the latency objective considers shapes with this share of peak throughput


def pick(results: list[dict], objective: str) -> dict:
    """throughput: the most bootstraps per second; latency: of the shapes within 15 % of that,
    the one that finishes a lone ciphertext soonest (what a serving loop under partial load
    sees)."""
    best = max(results, key=lambda r: r["bootstraps_per_s"])
    if objective == "throughput":
        return best
    near = [r for r in results if r["bootstraps_per_s"] >= LATENCY_WINDOW * best["bootstraps_per_s"]]
    return min(near, key=lambda r: r["single_ms"])


def tune(ctx, key, lut, count: int | None = None, use_cache: bool = True, verbose: bool = False,
         objective: str = "throughput") -> dict:
    """Picks, applies and caches the best launch shape for `objective`; returns
    {choice, results, cached}."""
    import torch

    if objective not in OBJECTIVES:
        raise ValueError(f"objective must be one of {OBJECTIVES}")
    k = _key(ctx) + f"|{objective}"
    table = _load() if use_cache else {}
    if k in table:
        c = table[k]
        api.set_launch(ctx, c["per_cta"], c["ctas_per_sm"], c.get("layout", 0))
        return {"choice": c, "cached": True}
    sms = torch.cuda.get_device_properties(ctx.device).multi_processor_count
    if count is None:
        count = sms * 16  # several waves for every candidate
    results = []
    for layout, per_cta, cps in candidates(ctx):
        bps, single = measure(ctx, key, lut, count, per_cta, cps, layout=layout)
        results.append({"layout": layout, "per_cta": per_cta, "ctas_per_sm": cps, "bootstraps_per_s": bps,
                        "single_ms": single})
        if verbose:
            print(f"autotune layout {layout}, {per_cta}/CTA, {cps or 'all'} CTAs/SM: {bps:.0f} bootstraps/s, "
                  f"{single:.2f} ms alone")
    best = pick(results, objective)
    table = _load()
    table[k] = {**best, "sample": count, "objective": objective}
    _store(table)
    api.set_launch(ctx, best["per_cta"], best["ctas_per_sm"], best["layout"])
    return {"choice": table[k], "results": results, "cached": False}

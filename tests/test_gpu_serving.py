"""GPU: the serving loop.  Requests from several tenants arrive while others run (continuous
batching) through an HBM key cache too small for all tenants (LRU refills from pinned host
memory); every output must equal the same computation done alone, which in turn equals
the oracle."""
import numpy as np
import pytest

from oracle.oracle import Restatement
from yatfhe_gb300 import lut as lutmod
from yatfhe_gb300.params import T32_N1024, small

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def served(built_lib):
    from yatfhe_gb300 import api, serving

    p = small(T32_N1024, 24)
    ctx = api.Context(p, 0)
    tenants, max_count = 6, 16
    oras, keys = [], []
    for t in range(tenants):
        o = Restatement(p)
        o.keygen(1000 + t)
        oras.append(o)
        keys.append(api.BootstrapKey.from_ntt_words(ctx, o.bsk_ntt()).set_ksk(o.ksk()))
    per_key = keys[0].device_bytes
    srv = serving.Server(ctx, key_budget_bytes=2.5 * per_key, max_batch=64, max_inflight=2)
    luts = [lutmod.sign_lut(p.N, 32), lutmod.box_lut(p.N, 32, np.arange(8) << 28)]
    pool = torch.empty((tenants, max_count, p.n + 1), dtype=torch.int32).pin_memory()
    expect = torch.empty_like(pool).pin_memory()
    rng = np.random.default_rng(3)
    for t in range(tenants):
        lut = luts[t % 2]
        srv.add_tenant(t, keys[t], lut)
        lwe = oras[t].encrypt(rng.integers(-(1 << 31), 1 << 31, max_count))
        pool[t] = torch.from_numpy(lwe)
        # the same computation alone: one call, this tenant's key and LUT only
        alone = api.functional_bootstrapping_mp_ntt(ctx, keys[t], torch.from_numpy(lwe).cuda(),
                                                    torch.from_numpy(lut).cuda()).cpu()
        expect[t] = alone
        if t < 2:
            np.testing.assert_array_equal(alone.numpy()[:4], oras[t].pbs(lwe[:4], lut))
    srv.start()
    yield ctx, srv, pool, expect
    srv.close()


def test_requests_alone_and_in_the_mix(served):
    ctx, srv, pool, expect = served
    outs = [torch.zeros((16, ctx.params.n + 1), dtype=torch.int32).pin_memory() for _ in range(12)]
    ids = [srv.submit(i % 6, pool[i % 6], outs[i], count=1 + (i * 5) % 16) for i in range(12)]
    for i, rid in enumerate(ids):
        t = srv.wait(rid)
        assert t["t_submit"] <= t["t_start"] <= t["t_done"]
        c = 1 + (i * 5) % 16
        assert torch.equal(outs[i][:c], expect[i % 6][:c]), f"request {i}"


def test_trace_with_evictions_is_bit_exact(served):
    ctx, srv, pool, expect = served
    res = srv.run_trace(pool, expect, requests=300, warmup=20, rate=2000.0, zipf_s=1.1, max_count=16, seed=7)
    assert res["served"] == 300
    assert res["mismatched_requests"] == 0
    assert res["key_misses"] > 0 and 0 < res["hit_rate"] < 1  # 2 of 6 tenants fit: refills happened
    assert res["sojourn"]["p50_ms"] > 0 and res["sojourn"]["p99_ms"] >= res["sojourn"]["p50_ms"]
    c = srv.counters()
    assert c["key_slots"] == 2
    # the reference harness's figures: SLO violation shares, Jain's index over the tenants'
    # mean sojourn (1 / tenants <= J <= 1), peak queue depth, refills in flight
    assert res["slo_ms"] == 100.0
    for k in ("slo_violation_rate", "slo_violation_rate_100", "slo_violation_rate_300", "slo_violation_rate_500"):
        assert 0.0 <= res[k] <= 1.0
    assert res["slo_violation_rate"] == res["slo_violation_rate_100"]
    assert res["slo_violation_rate_100"] >= res["slo_violation_rate_300"] >= res["slo_violation_rate_500"]
    assert 1.0 / 6 - 1e-9 <= res["tenant_fairness_jain"] <= 1.0 + 1e-9
    assert res["peak_queue_depth"] >= 1
    assert 1 <= res["load_concurrency_peak"] and 0.0 < res["load_concurrency_mean"] <= res["load_concurrency_peak"]
    tight = srv.run_trace(pool, expect, requests=60, warmup=0, rate=2000.0, zipf_s=1.1, max_count=16, seed=8,
                          slo_ms=1e-6)
    assert tight["slo_violation_rate"] == 1.0  # every sojourn exceeds a near-zero target
    # small batches ran in the channel-cluster layout (the default: two waves of its clusters)
    assert 0 < res["latency_batches"] <= res["batches"]


def test_latency_layout_off_and_forced(built_lib):
    """The same trace with the latency layout off (negative latency_batch_max) and forced for
    every batch (a bound above max_batch) gives the same bit-exact outputs; only the
    batches' layout differs."""
    from yatfhe_gb300 import api, serving

    p = small(T32_N1024, 24)
    ctx = api.Context(p, 0)
    tenants, max_count = 3, 16
    keys = []
    pool = torch.empty((tenants, max_count, p.n + 1), dtype=torch.int32).pin_memory()
    expect = torch.empty_like(pool).pin_memory()
    lut = lutmod.sign_lut(p.N, 32)
    rng = np.random.default_rng(8)
    for t in range(tenants):
        o = Restatement(p)
        o.keygen(2000 + t)
        keys.append(api.BootstrapKey.from_ntt_words(ctx, o.bsk_ntt()).set_ksk(o.ksk()))
        lwe = o.encrypt(rng.integers(-(1 << 31), 1 << 31, max_count))
        pool[t] = torch.from_numpy(lwe)
        expect[t] = api.functional_bootstrapping_mp_ntt(ctx, keys[t], torch.from_numpy(lwe).cuda(),
                                                        torch.from_numpy(lut).cuda()).cpu()
    for bound, want in ((-1, "none"), (1 << 20, "all")):
        srv = serving.Server(ctx, key_budget_bytes=4 * keys[0].device_bytes, max_batch=48, max_inflight=2,
                             latency_batch_max=bound)
        for t in range(tenants):
            srv.add_tenant(t, keys[t], lut)
        srv.start()
        res = srv.run_trace(pool, expect, requests=120, warmup=10, rate=3000.0, max_count=max_count, seed=9)
        srv.close()
        assert res["mismatched_requests"] == 0 and res["served"] == 120
        assert res["latency_batches"] == (0 if want == "none" else res["batches"])


def test_trace_sheds_beyond_queue_bound(served):
    """queue_max: arrivals that find more unfinished requests than the bound are shed (the
    reference's shed at queueMax); what is served stays bit-exact."""
    ctx, srv, pool, expect = served
    res = srv.run_trace(pool, expect, requests=200, warmup=0, rate=1e6, zipf_s=1.1, max_count=16, seed=9,
                        queue_max=4)
    assert res["shed"] > 0
    assert res["served"] + res["shed"] == 200
    assert res["mismatched_requests"] == 0

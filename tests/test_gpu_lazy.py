"""GPU tests of the lazy ("OURS") key family: the lazy blind rotation (lazy_blind_rotate_kernel,
blindRotateLazyPipeAltNtt) gives the reference's bootstrap outputs and accumulators bit for bit
(golden fixtures from the reference's own code on its default sets), equals the restatement on
random ciphertexts and test polynomials (including skipped steps), loads the reference's file
format, and is refused by the entry points that only take GINX rows."""
import hashlib
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import Restatement
from yatfhe_gb300.params import PbsParams, WWL24_T32_N2048, WWL24_T56_N2048, small

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def _sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _random_case(p, count, seed):
    rng = np.random.default_rng(seed)
    lwe = rng.integers(-(1 << 31), 1 << 31, size=(count, p.n + 1), dtype=np.int64).astype(np.int32)
    lwe[1, : p.n // 2] = 0          # half the CMux steps skipped (a_i = 0)
    lwe[2, :] = 0                   # every step skipped, a_0 = b = 0
    lwe[3, 0] = 1 << 30             # a_0 = N / 2 after the modulus switch
    lut = rng.integers(-(1 << (p.torus_bits - 1)), 1 << (p.torus_bits - 1), size=p.N, dtype=np.int64)
    return lwe, lut


@pytest.mark.parametrize("name", ["lazy_t32_n2048_seed5eed0007", "lazy_t56_n2048_seed5eed0008"])
def test_gpu_reproduces_reference_lazy_golden(name, built_lib):
    from yatfhe_gb300 import api

    g = np.load(GOLDEN / f"{name}.npz")
    p = PbsParams(*[int(x) for x in g["params"]])
    ora = Restatement(p)
    ora.keygen_lazy(int(g["seed"][0]))
    cprime, s2 = ora.lazy_words()
    assert _sha(cprime) == str(g["sha_cprime"]) and _sha(s2) == str(g["sha_s2"])  # the reference's keys
    ctx = api.Context(p, 0)
    key = api.BootstrapKey.from_lazy_words(ctx, cprime, s2).set_ksk(ora.ksk())
    d_in = torch.from_numpy(g["lwe_in"]).cuda()
    d_lut = torch.from_numpy(g["lut"]).cuda()
    out = api.functional_bootstrapping_mp_ntt(ctx, key, d_in, d_lut).cpu().numpy()
    np.testing.assert_array_equal(out, g["lwe_out"])
    np.testing.assert_array_equal(ora.decrypt(out, int(g["base"][0])), g["decrypted"])
    acc = api.blind_rotate_lazy_pipe_alt_ntt(ctx, key, d_in[:1], d_lut).cpu().numpy()[0]
    np.testing.assert_array_equal(acc.reshape(-1), g["acc0"])
    # the device keeps the rows in the torus word size, beside the s2 key and transform tables
    word = 4 if p.torus_bits == 32 else 8
    assert key.device_bytes == cprime.size * word + 2 * s2.nbytes + 4 * 8 * p.N + p.ksk_words * 4


@pytest.mark.parametrize("base", [WWL24_T32_N2048, WWL24_T56_N2048])
def test_gpu_lazy_equals_restatement_on_random_inputs(base, built_lib):
    """64 random ciphertexts and a random test polynomial at n = 12: accumulators and outputs
    equal the restatement's."""
    from yatfhe_gb300 import api

    p = small(base, 12)
    ora = Restatement(p)
    ora.keygen_lazy(31)
    cprime, s2 = ora.lazy_words()
    ctx = api.Context(p, 0)
    key = api.BootstrapKey.from_lazy_words(ctx, cprime, s2).set_ksk(ora.ksk())
    lwe, lut = _random_case(p, 64, 7)
    d_in, d_lut = torch.from_numpy(lwe).cuda(), torch.from_numpy(lut).cuda()
    acc = api.blind_rotate_lazy_pipe_alt_ntt(ctx, key, d_in, d_lut).cpu().numpy()
    for c in (0, 1, 2, 3, 63):
        np.testing.assert_array_equal(acc[c], ora.blind_rotate_lazy(lwe[c], lut), err_msg=f"ciphertext {c}")
    out = api.functional_bootstrapping_mp_ntt(ctx, key, d_in, d_lut).cpu().numpy()
    np.testing.assert_array_equal(out, ora.pbs_lazy(lwe, lut, threads=8))


def test_gpu_lazy_file_host_buffers_and_refusals(tmp_path, built_lib):
    from yatfhe_gb300 import api

    p = small(WWL24_T32_N2048, 9)
    ora = Restatement(p)
    ora.keygen_lazy(8)
    ora.save_lazy_file(tmp_path / "k.bin")
    cprime, s2 = ora.lazy_words()
    ctx = api.Context(p, 0)
    kf = api.BootstrapKey.from_lazy_file(ctx, tmp_path / "k.bin").set_ksk(ora.ksk())
    kw = api.BootstrapKey.from_lazy_words(ctx, cprime, s2).set_ksk(ora.ksk())
    lwe, lut = _random_case(p, 40, 9)
    d_in, d_lut = torch.from_numpy(lwe).cuda(), torch.from_numpy(lut).cuda()
    a = api.functional_bootstrapping_mp_ntt(ctx, kf, d_in, d_lut).cpu().numpy()
    b = api.functional_bootstrapping_mp_ntt_host(ctx, kw, lwe, lut)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, ora.pbs_lazy(lwe, lut, threads=8))
    # a plan takes keys of one family
    og = Restatement(p)
    og.keygen(8)
    kg = api.BootstrapKey.from_ntt_words(ctx, og.bsk_ntt()).set_ksk(og.ksk())
    with pytest.raises(ValueError, match="one family"):
        api.BatchPlan(ctx, [kw, kg], [d_lut], 4, key_ids=[0, 0, 1, 1])
    with pytest.raises(ValueError, match="steps = n"):
        api.blind_rotate_mp21_ntt(ctx, kw, d_in, d_lut, steps=3)
    # a row word that is not a sign-extended torus value
    bad = cprime.copy()
    bad[0, 0, 0, 0] = 1 << 40
    with pytest.raises(ValueError, match="sign-extended"):
        api.BootstrapKey.from_lazy_words(ctx, bad, s2)
    # a WWL+24 key file is not a lazy key file
    ow = Restatement(p)
    ow.keygen_wwl24(8)
    ow.save_wwl24_file(tmp_path / "w.bin")
    with pytest.raises(OSError, match="expected"):
        api.BootstrapKey.from_lazy_file(ctx, tmp_path / "w.bin")


def _lazy_tenants(p, seeds):
    from yatfhe_gb300 import api

    ctx = api.Context(p, 0)
    oras, keys = [], []
    for sd in seeds:
        o = Restatement(p)
        o.keygen_lazy(sd)
        cprime, s2 = o.lazy_words()
        oras.append(o)
        keys.append(api.BootstrapKey.from_lazy_words(ctx, cprime, s2).set_ksk(o.ksk()))
    return ctx, oras, keys


def test_lazy_keys_in_a_multi_key_plan(built_lib):
    """Several lazy keys and test polynomials in one launch pair (yg_plan_*, the lazy blind
    rotation reading a per-ciphertext key table): every output equals the same ciphertext
    bootstrapped alone under its own key, which equals the restatement."""
    from yatfhe_gb300 import api

    p = small(WWL24_T32_N2048, 9)
    ctx, oras, keys = _lazy_tenants(p, [41, 42, 43])
    rng = np.random.default_rng(4)
    counts = [5, 1, 12]
    key_ids = np.concatenate([np.full(c, t, np.int32) for t, c in enumerate(counts)])
    lwe = np.concatenate([_random_case(p, max(c, 4), 50 + t)[0][:c] for t, c in enumerate(counts)])
    luts_np = [_random_case(p, 4, 60)[1], _random_case(p, 4, 61)[1]]
    lut_ids = rng.integers(0, 2, len(lwe)).astype(np.int32)
    luts = [torch.from_numpy(v).cuda() for v in luts_np]
    d_in = torch.from_numpy(lwe).cuda()
    plan = api.BatchPlan(ctx, keys, luts, len(lwe), key_ids=key_ids, lut_ids=lut_ids)
    got = plan.run(d_in, torch.empty_like(d_in)).cpu().numpy()
    torch.cuda.synchronize()
    for c in range(len(lwe)):
        alone = api.functional_bootstrapping_mp_ntt(ctx, keys[key_ids[c]], d_in[c:c + 1], luts[lut_ids[c]])
        np.testing.assert_array_equal(got[c], alone.cpu().numpy()[0], err_msg=f"ciphertext {c}")
    for c in (0, 5, 6):
        np.testing.assert_array_equal(got[c:c + 1], oras[key_ids[c]].pbs_lazy(lwe[c:c + 1], luts_np[lut_ids[c]], threads=8))


def test_serving_lazy_tenants(built_lib):
    """The serving loop with lazy keys: a lazy server's HBM slots hold the half rows and the s2
    key (a third of the GINX rows' bytes at this set), so the same budget holds more tenants;
    a trace with evictions returns every output equal to the same ciphertexts bootstrapped
    alone."""
    from yatfhe_gb300 import api, serving

    p = small(WWL24_T32_N2048, 9)
    tenants, max_count = 6, 8
    ctx, oras, keys = _lazy_tenants(p, [70 + t for t in range(tenants)])
    og = Restatement(p)
    og.keygen(70)
    ginx = api.BootstrapKey.from_ntt_words(ctx, og.bsk_ntt()).set_ksk(og.ksk())
    budget = 2.5 * keys[0].device_bytes
    srv = serving.Server(ctx, key_budget_bytes=budget, max_batch=32, max_inflight=2)
    pool = torch.empty((tenants, max_count, p.n + 1), dtype=torch.int32).pin_memory()
    expect = torch.empty_like(pool).pin_memory()
    for t in range(tenants):
        lwe, lut = _random_case(p, max_count, 80 + t)
        srv.add_tenant(t, keys[t], lut)
        pool[t] = torch.from_numpy(lwe)
        expect[t] = api.functional_bootstrapping_mp_ntt(ctx, keys[t], torch.from_numpy(lwe).cuda(),
                                                        torch.from_numpy(lut).cuda()).cpu()
    with pytest.raises(ValueError, match="one family"):
        srv.add_tenant(tenants, ginx, lut)
    srv.start()
    res = srv.run_trace(pool, expect, requests=120, warmup=0, rate=2000.0, zipf_s=1.1, max_count=max_count, seed=5)
    c = srv.counters()
    srv.close()
    assert res["served"] == 120 and res["mismatched_requests"] == 0
    assert c["key_slots"] == 2 and res["key_misses"] > 0
    # the same budget holds fewer GINX tenants (their rows take three times the bytes)
    assert int(budget // ginx.device_bytes) < c["key_slots"]

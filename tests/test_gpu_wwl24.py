"""GPU tests of the WWL+24 key family: the GINX rows derived on the GPU at upload
(wwl24_expand_kernel) give the reference's bootstrap outputs and accumulators bit for bit
(golden fixtures from the reference's blindRotateWWL24Ntt), equal the rows the restatement
derives, and the reference's file format loads."""
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


@pytest.mark.parametrize("name", ["wwl24_t32_n2048_seed5eed0005", "wwl24_t56_n2048_seed5eed0006"])
def test_gpu_reproduces_reference_wwl24_golden(name, built_lib):
    from yatfhe_gb300 import api

    g = np.load(GOLDEN / f"{name}.npz")
    p = PbsParams(*[int(x) for x in g["params"]])
    ora = Restatement(p)
    ora.keygen_wwl24(int(g["seed"][0]))
    cprime, s2 = ora.wwl24_words()
    assert _sha(cprime) == str(g["sha_cprime"]) and _sha(s2) == str(g["sha_s2"])  # the reference's keys
    ctx = api.Context(p, 0)
    key = api.BootstrapKey.from_wwl24_words(ctx, cprime, s2).set_ksk(ora.ksk())
    d_in = torch.from_numpy(g["lwe_in"]).cuda()
    d_lut = torch.from_numpy(g["lut"]).cuda()
    out = api.functional_bootstrapping_mp_ntt(ctx, key, d_in, d_lut).cpu().numpy()
    np.testing.assert_array_equal(out, g["lwe_out"])
    np.testing.assert_array_equal(ora.decrypt(out, int(g["base"][0])), g["decrypted"])
    acc = api.blind_rotate_wwl24_ntt(ctx, key, d_in[:1], d_lut).cpu().numpy()[0]
    np.testing.assert_array_equal(acc.reshape(-1), g["acc0"])


@pytest.mark.parametrize("base", [WWL24_T32_N2048, WWL24_T56_N2048])
def test_gpu_wwl24_rows_equal_restatement(base, built_lib):
    """The key derived on the GPU and the restatement's derived rows uploaded as a GINX key give
    the same accumulators on 96 random ciphertexts (every key row enters them)."""
    from yatfhe_gb300 import api

    p = base
    ora = Restatement(p)
    ora.keygen_wwl24(77)
    cprime, s2 = ora.wwl24_words()
    ctx = api.Context(p, 0)
    kw = api.BootstrapKey.from_wwl24_words(ctx, cprime, s2)
    kg = api.BootstrapKey.from_ntt_words(ctx, ora.wwl24_expanded())
    rng = np.random.default_rng(4)
    lwe = rng.integers(-(1 << 31), 1 << 31, size=(96, p.n + 1), dtype=np.int64).astype(np.int32)
    lut = rng.integers(-(1 << (p.torus_bits - 1)), 1 << (p.torus_bits - 1), size=p.N, dtype=np.int64)
    d_in, d_lut = torch.from_numpy(lwe).cuda(), torch.from_numpy(lut).cuda()
    a = api.blind_rotate_wwl24_ntt(ctx, kw, d_in, d_lut).cpu().numpy()
    b = api.blind_rotate_mp21_ntt(ctx, kg, d_in, d_lut).cpu().numpy()
    np.testing.assert_array_equal(a, b)
    _, ref0 = ora.blind_rotate_trace(lwe[0], lut, [])
    np.testing.assert_array_equal(a[0].reshape(-1), ref0)


def test_gpu_wwl24_file_and_errors(tmp_path, built_lib):
    from yatfhe_gb300 import api

    p = small(WWL24_T32_N2048, 7)
    ora = Restatement(p)
    ora.keygen_wwl24(8)
    ora.save_wwl24_file(tmp_path / "k.bin")
    cprime, s2 = ora.wwl24_words()
    ctx = api.Context(p, 0)
    kf = api.BootstrapKey.from_wwl24_file(ctx, tmp_path / "k.bin")
    kw = api.BootstrapKey.from_wwl24_words(ctx, cprime, s2)
    rng = np.random.default_rng(6)
    lwe = rng.integers(-(1 << 31), 1 << 31, size=(16, p.n + 1), dtype=np.int64).astype(np.int32)
    lut = rng.integers(-(1 << 31), 1 << 31, size=p.N, dtype=np.int64)
    d_in, d_lut = torch.from_numpy(lwe).cuda(), torch.from_numpy(lut).cuda()
    np.testing.assert_array_equal(api.blind_rotate_wwl24_ntt(ctx, kf, d_in, d_lut).cpu().numpy(),
                                  api.blind_rotate_wwl24_ntt(ctx, kw, d_in, d_lut).cpu().numpy())
    with pytest.raises(ValueError):
        api.blind_rotate_wwl24_ntt(ctx, api.BootstrapKey.from_ntt_words(ctx, ora.wwl24_expanded()), d_in, d_lut)
    bad = s2.copy()
    bad.reshape(-1)[5] = p.q_ntt
    with pytest.raises(ValueError):
        api.BootstrapKey.from_wwl24_words(ctx, cprime, bad)
    bad = cprime.copy()
    bad.reshape(-1)[9] = p.q_ntt
    with pytest.raises(ValueError):
        api.BootstrapKey.from_wwl24_words(ctx, bad, s2)
    raw = (tmp_path / "k.bin").read_bytes()
    (tmp_path / "short.bin").write_bytes(raw[:-64])
    with pytest.raises(Exception):
        api.BootstrapKey.from_wwl24_file(ctx, tmp_path / "short.bin")


def test_serving_mixes_wwl24_and_ginx_tenants(built_lib):
    """yg_server_add_tenant snapshots any key handle: WWL+24 tenants (rows derived at upload)
    and GINX tenants share the HBM key cache, evictions included, bit-exact."""
    from yatfhe_gb300 import api, serving
    from yatfhe_gb300 import lut as lutmod

    p = small(WWL24_T32_N2048, 10)
    ctx = api.Context(p, 0)
    keys = []
    for t in range(4):
        o = Restatement(p)
        if t % 2:
            o.keygen_wwl24(500 + t)
            keys.append(api.BootstrapKey.from_wwl24_words(ctx, *o.wwl24_words()).set_ksk(o.ksk()))
        else:
            o.keygen(500 + t)
            keys.append(api.BootstrapKey.from_ntt_words(ctx, o.bsk_ntt()).set_ksk(o.ksk()))
    srv = serving.Server(ctx, key_budget_bytes=1.5 * keys[0].device_bytes, max_batch=32, max_inflight=2)
    lut = lutmod.sign_lut(p.N, 32)
    rng = np.random.default_rng(12)
    pool = torch.empty((4, 8, p.n + 1), dtype=torch.int32).pin_memory()
    expect = torch.empty_like(pool).pin_memory()
    for t in range(4):
        srv.add_tenant(t, keys[t], lut)
        lwe = rng.integers(-(1 << 31), 1 << 31, size=(8, p.n + 1), dtype=np.int64).astype(np.int32)
        pool[t] = torch.from_numpy(lwe)
        expect[t] = api.functional_bootstrapping_mp_ntt(ctx, keys[t], torch.from_numpy(lwe).cuda(),
                                                        torch.from_numpy(lut).cuda()).cpu()
    srv.start()
    try:
        res = srv.run_trace(pool, expect, requests=60, warmup=0, rate=500.0, zipf_s=1.1, max_count=8, seed=3)
        assert res["served"] == 60 and res["mismatched_requests"] == 0
        assert res["key_misses"] > 0
    finally:
        srv.close()

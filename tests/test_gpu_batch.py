"""GPU: batches under several keys and LUTs in one launch pair (yg_plan_*), persistent
grids, CUDA-graph replay, and the key-file entry point; every output bit-exact against the
oracle run one tenant at a time."""
import numpy as np
import pytest

from oracle.oracle import Restatement
from yatfhe_gb300 import lut as lutmod
from yatfhe_gb300.params import T32_N1024, T56_N2048, small

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _tenants(p, seeds):
    from yatfhe_gb300 import api

    ctx = api.Context(p, 0)
    oras, keys = [], []
    for s in seeds:
        o = Restatement(p)
        o.keygen(s)
        oras.append(o)
        keys.append(api.BootstrapKey.from_ntt_words(ctx, o.bsk_ntt()).set_ksk(o.ksk()))
    return ctx, oras, keys


@pytest.mark.parametrize("base", [T32_N1024, T56_N2048])
def test_multi_key_batch_matches_per_tenant_oracle(base, built_lib):
    from yatfhe_gb300 import api

    p = small(base, 10)
    ctx, oras, keys = _tenants(p, [101, 102, 103])
    rng = np.random.default_rng(1)
    counts = [7, 1, 12]  # uneven, with a run of 12 > one key-switch tile
    key_ids = np.concatenate([np.full(c, t, np.int32) for t, c in enumerate(counts)])
    T = p.torus_bits
    luts_np = [lutmod.sign_lut(p.N, T), lutmod.box_lut(p.N, T, rng.integers(-8, 8, 8) << (T - 4))]
    lut_ids = rng.integers(0, 2, len(key_ids)).astype(np.int32)
    lwe = np.concatenate([oras[t].encrypt(rng.integers(-(1 << 31), 1 << 31, c)) for t, c in enumerate(counts)])
    luts = [torch.from_numpy(v).cuda() for v in luts_np]
    d_in = torch.from_numpy(lwe).cuda()
    shapes = [(lay, g, grid) for lay in (0, 1, 2) for g in (1, 2, 4) if api.ctas_per_sm(ctx, g, lay) > 0
              for grid in (0, 3)]
    assert (0, 1, 0) in shapes and (1, 1, 0) in shapes
    assert (0, 2, 0) in shapes or p.N == 2048
    assert ((2, 1, 0) in shapes) == (p.torus_bits == 32 and p.N == 1024)  # the row-cluster layout
    for lay, g in ((0, 4), (1, 4), (2, 2)):
        if api.ctas_per_sm(ctx, g, lay) == 0:  # no such kernel or too large: rejected, never skipped
            with pytest.raises(ValueError):
                api.BatchPlan(ctx, keys, luts, len(lwe), key_ids=key_ids, lut_ids=lut_ids, per_cta=g, layout=lay)
    want = np.concatenate([oras[key_ids[c]].pbs(lwe[c:c + 1], luts_np[lut_ids[c]]) for c in range(len(lwe))])
    for layout, per_cta, grid in shapes:
        plan = api.BatchPlan(ctx, keys, luts, len(lwe), key_ids=key_ids, lut_ids=lut_ids, grid=grid, per_cta=per_cta,
                             layout=layout)
        out = plan.run(d_in, torch.empty_like(d_in))
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), want, err_msg=f"layout {layout}, {per_cta}/CTA, grid {grid}")


def test_plan_replays_in_a_cuda_graph(built_lib):
    from yatfhe_gb300 import api

    p = small(T32_N1024, 12)
    ctx, oras, keys = _tenants(p, [7])
    lut = torch.from_numpy(lutmod.sign_lut(p.N, 32)).cuda()
    mu = np.array([(1 if i % 2 else -1) << 29 for i in range(40)], np.int64)
    lwe = oras[0].encrypt(mu)
    d_in = torch.from_numpy(lwe).cuda()
    d_out = torch.empty_like(d_in)
    plan = api.BatchPlan(ctx, keys, [lut], len(lwe), grid=16)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        plan.run(d_in, d_out, stream=s)  # warm up (per-device kernel set-up happens here)
    s.synchronize()
    d_out.zero_()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.run(d_in, d_out, stream=s)
    for _ in range(2):
        d_out.zero_()
        g.replay()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(d_out.cpu().numpy(), oras[0].pbs(lwe, lut.cpu().numpy(), threads=8))


def test_key_file_entry_point(tmp_path, built_lib):
    """yg_key_load_bsk_file reads the reference's serializeBskMP format."""
    from yatfhe_gb300 import api

    p = small(T56_N2048, 6)
    ora = Restatement(p)
    ora.keygen(55)
    f = tmp_path / "BSK_GINX_1.bin"
    ora.save_bsk_file(f)
    ctx = api.Context(p, 0)
    key = api.BootstrapKey.from_file(ctx, f).set_ksk(ora.ksk())
    lwe = ora.encrypt(np.array([0, 1 << 27, 5 << 27], np.int64))
    lut = lutmod.padded_message_lut(p.N, 56, np.arange(16)[::-1])
    got = api.functional_bootstrapping_mp_ntt(ctx, key, torch.from_numpy(lwe).cuda(),
                                              torch.from_numpy(lut).cuda()).cpu().numpy()
    np.testing.assert_array_equal(got, ora.pbs(lwe, lut))
    with pytest.raises(OSError):
        api.BootstrapKey.from_file(ctx, tmp_path / "missing.bin")
    (tmp_path / "short.bin").write_bytes(f.read_bytes()[:1000])
    with pytest.raises(OSError):
        api.BootstrapKey.from_file(ctx, tmp_path / "short.bin")

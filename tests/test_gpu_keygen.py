"""GPU key generation from caller-drawn samples (yg_keygen_from_samples): fed the random
samples of the seeded key generation (the restatement's draws, in the reference's order),
the GPU makes the same keys bit for bit -- the reference's own, for the golden seed -- and
the key bootstraps like the uploaded one."""
import hashlib
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import Restatement
from yatfhe_gb300 import lut as lutmod
from yatfhe_gb300.params import PbsParams, T32_N1024, T56_N2048, small

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def _sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("base,n", [(T32_N1024, 6), (T56_N2048, 4)])
def test_gpu_keygen_equals_restatement(base, n, built_lib):
    from yatfhe_gb300 import api

    p = small(base, n)
    ora = Restatement(p)
    smp = ora.keygen_samples(31)
    ctx = api.Context(p, 0)
    key, words, ksk = api.keygen_from_samples(ctx, smp, return_keys=True)
    np.testing.assert_array_equal(words, ora.bsk_ntt())
    np.testing.assert_array_equal(ksk, ora.ksk())
    rng = np.random.default_rng(2)
    mu = np.where(rng.integers(0, 2, 6) == 1, 1 << 29, -(1 << 29)).astype(np.int64)
    lwe = ora.encrypt(mu)
    lut = lutmod.sign_lut(p.N, p.torus_bits)
    out = api.functional_bootstrapping_mp_ntt(ctx, key, torch.from_numpy(lwe).cuda(), torch.from_numpy(lut).cuda())
    np.testing.assert_array_equal(out.cpu().numpy(), ora.pbs(lwe, lut))


def test_gpu_keygen_reproduces_reference_keys(built_lib):
    """Golden key digests: the reference's own keys for seed 0x5EED0001 at n = 630."""
    from yatfhe_gb300 import api

    g = np.load(GOLDEN / "t32_n1024_seed5eed0001.npz")
    p = PbsParams(*[int(x) for x in g["params"]])
    smp = Restatement(p).keygen_samples(int(g["seed"][0]))
    ctx = api.Context(p, 0)
    key, words, ksk = api.keygen_from_samples(ctx, smp, return_keys=True)
    assert _sha(words) == str(g["sha_bsk"]) and _sha(ksk) == str(g["sha_ksk"])
    out = api.functional_bootstrapping_mp_ntt(ctx, key, torch.from_numpy(g["lwe_in"]).cuda(),
                                              torch.from_numpy(g["lut"]).cuda())
    np.testing.assert_array_equal(out.cpu().numpy(), g["lwe_out"])


def test_gpu_keygen_rejects_bad_samples(built_lib):
    from yatfhe_gb300 import api

    p = small(T32_N1024, 3)
    smp = Restatement(p).keygen_samples(5)
    ctx = api.Context(p, 0)
    bad = dict(smp, lwe_s=smp["lwe_s"].copy())
    bad["lwe_s"][1] = 2
    with pytest.raises(ValueError):
        api.keygen_from_samples(ctx, bad)
    bad = dict(smp, bsk_mask=smp["bsk_mask"].copy())
    bad["bsk_mask"].reshape(-1)[17] = p.q_ntt
    with pytest.raises(ValueError):
        api.keygen_from_samples(ctx, bad)

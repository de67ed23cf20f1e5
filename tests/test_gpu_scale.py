"""GPU parity at batch scale (full T32 set, n = 630, N = 1024): 4,864 sign bootstraps in one
call (32 ciphertexts per SM of a 152-SM GB300, so every CTA of the tuned persistent grid runs
many ciphertexts), each output decrypted with the LWE secret and compared with its sign, a
sample from every part of the batch compared bit for bit with the oracle, and the same batch
in every other layout equal to the first bit for bit."""
import numpy as np
import pytest

from oracle.oracle import Restatement
from yatfhe_gb300 import lut as lutmod
from yatfhe_gb300.params import T32_N1024

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

COUNT = 4864


def test_batch_scale_decrypts_and_matches(built_lib):
    from yatfhe_gb300 import api

    p = T32_N1024
    ora = Restatement(p)
    ora.keygen(0x5EED0001)
    ctx = api.Context(p, 0)
    key = api.BootstrapKey.from_ntt_words(ctx, ora.bsk_ntt()).set_ksk(ora.ksk())
    rng = np.random.default_rng(0x5CA1E)
    bits = rng.integers(0, 2, COUNT)
    mu = np.where(bits == 1, 1 << 29, -(1 << 29)).astype(np.int64)
    lwe = ora.encrypt(mu)
    lut = lutmod.sign_lut(p.N, 32)
    d_in, d_lut = torch.from_numpy(lwe).cuda(), torch.from_numpy(lut).cuda()
    outs = {}
    for layout, per_cta, ctas_per_sm in ((1, 2, 1), (0, 4, 0), (1, 1, 0), (2, 1, 0), (3, 1, 0)):
        if api.ctas_per_sm(ctx, per_cta, layout) < 1:
            continue
        api.set_launch(ctx, per_cta, ctas_per_sm, layout)
        outs[(layout, per_cta, ctas_per_sm)] = api.functional_bootstrapping_mp_ntt(ctx, key, d_in, d_lut).cpu().numpy()
    api.set_launch(ctx, 1, 0, 0)
    first = next(iter(outs.values()))
    for shape, got in outs.items():
        np.testing.assert_array_equal(got, first, err_msg=f"layout, per_cta, ctas_per_sm = {shape}")
    np.testing.assert_array_equal(ora.decrypt(first, 8), np.where(bits == 1, 1, -1))
    sample = np.unique(np.concatenate([np.arange(8), rng.integers(0, COUNT, 16), np.arange(COUNT - 8, COUNT)]))
    np.testing.assert_array_equal(first[sample], ora.pbs(lwe[sample], lut, threads=16))

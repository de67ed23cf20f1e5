"""GPU against the reference's own outputs: the golden fixtures in tests/golden/ were made by
the reference's sources (built against the HEXL/GMP stand-ins, tests/golden/make_golden.py).
The keys are regenerated from the recorded seed by the restatement, checked against the
reference's key digests, and handed to the CUDA path; its bootstrap outputs and its
accumulators at the recorded CMux checkpoints must equal the reference's bit for bit."""
import hashlib
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import Restatement
from yatfhe_gb300.params import PbsParams

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def _sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("layout", [0, 1, 2, 3])
@pytest.mark.parametrize("name", ["t32_n1024_small40_seed7", "t32_n1024_seed5eed0001", "t56_n2048_seed5eed0003"])
def test_gpu_reproduces_reference_golden(name, layout, built_lib):
    """Every layout of the blind rotation (channel, channel-row, and the row- and
    channel-cluster layouts where they exist)."""
    from yatfhe_gb300 import api

    g = np.load(GOLDEN / f"{name}.npz")
    p = PbsParams(*[int(x) for x in g["params"]])
    ora = Restatement(p)
    ora.keygen(int(g["seed"][0]))
    bsk, ksk = ora.bsk_ntt(), ora.ksk()
    assert _sha(bsk) == str(g["sha_bsk"]) and _sha(ksk) == str(g["sha_ksk"])  # the reference's keys
    ctx = api.Context(p, 0)
    if api.ctas_per_sm(ctx, 1, layout) < 1:
        assert layout in (2, 3) and not (p.torus_bits == 32 and p.N == 1024)
        pytest.skip("no cluster kernel for this parameter set")
    api.set_launch(ctx, 1, 0, layout)
    key = api.BootstrapKey.from_ntt_words(ctx, bsk).set_ksk(ksk)
    d_in = torch.from_numpy(g["lwe_in"]).cuda()
    d_lut = torch.from_numpy(g["lut"]).cuda()
    out = api.functional_bootstrapping_mp_ntt(ctx, key, d_in, d_lut).cpu().numpy()
    np.testing.assert_array_equal(out, g["lwe_out"])
    np.testing.assert_array_equal(ora.decrypt(out, int(g["base"][0])), g["decrypted"])
    for k, step in enumerate(g["checkpoints"]):
        acc = api.blind_rotate_mp21_ntt(ctx, key, d_in[:1], d_lut, steps=int(step) + 1).cpu().numpy()[0]
        np.testing.assert_array_equal(acc, g["acc"][k], err_msg=f"accumulator after CMux step {step}")

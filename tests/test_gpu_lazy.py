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
    # entry points that take GINX rows only
    with pytest.raises(ValueError, match="keys run through"):
        api.BatchPlan(ctx, [kw], [d_lut], 4)
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

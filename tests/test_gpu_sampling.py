"""Randomness drawn on the GPU and LWE encryption on the GPU.

* symEncTlwe (yatfhe/src/tlwe.cpp:21-31) fed the restatement's masks and noise (drawn in the
  reference's order) gives its ciphertexts bit for bit, at both torus widths;
* yg_keygen(seed) equals yg_keygen_from_samples fed yg_draw_keygen_samples(seed), and the
  restatement bootstraps with the downloaded keys exactly as the GPU does with yg_keygen's;
* ciphertexts encrypted on the GPU under a GPU-made key bootstrap and decrypt correctly;
* the draws are deterministic in the seed and have the reference's distributions (binary
  secrets, TUniform(b) per genTUniformNoise, yatfhe/src/numeric.cpp:47-55, uniform masks).
"""
import numpy as np
import pytest

from oracle.oracle import Restatement
from yatfhe_gb300 import lut as lutmod
from yatfhe_gb300.params import T32_N1024, T56_N2048, small

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("base,n", [(T32_N1024, 630), (T56_N2048, 17)])
def test_encrypt_from_samples_matches_restatement(base, n, built_lib):
    from yatfhe_gb300 import api

    p = small(base, n)
    ora = Restatement(p)
    ora.keygen(7)
    lwe_s, _ = ora.keys()
    rng = np.random.default_rng(5)
    mu = rng.integers(-(1 << 31), 1 << 31, 300, dtype=np.int64)
    want, mask, noise = ora.encrypt_samples(mu)
    ctx = api.Context(p, 0)
    got = api.sym_enc_tlwe_from_samples(ctx, torch.from_numpy(lwe_s).cuda(), torch.from_numpy(mu).cuda(),
                                        torch.from_numpy(mask).cuda(), torch.from_numpy(noise).cuda())
    np.testing.assert_array_equal(got.cpu().numpy(), want)


def test_keygen_equals_keygen_from_its_draws(built_lib):
    from yatfhe_gb300 import api

    p = small(T32_N1024, 24)
    ctx = api.Context(p, 0)
    key, lwe_s, rlwe_s = api.keygen(ctx, 0xC0FFEE, p.lwe_noise_b, p.rlwe_noise_b, return_secrets=True)
    smp = api.draw_keygen_samples(ctx, 0xC0FFEE, p.lwe_noise_b, p.rlwe_noise_b)
    np.testing.assert_array_equal(smp["lwe_s"], lwe_s)
    np.testing.assert_array_equal(smp["rlwe_s"], rlwe_s)
    key2, words, ksk = api.keygen_from_samples(ctx, smp, return_keys=True)
    # the restatement on the downloaded keys bootstraps like the GPU on yg_keygen's key
    ora = Restatement(p)
    ora.set_keys(lwe_s, rlwe_s)
    ora.set_bsk_ntt(words)
    ora.set_ksk(ksk)
    mu = np.array([(m % 4) << 29 for m in range(64)], np.int64)
    lwe = api.sym_enc_tlwe(ctx, torch.from_numpy(lwe_s).cuda(), torch.from_numpy(mu).cuda(), 3, 0, p.lwe_noise_b)
    lut = lutmod.padded_message_lut(p.N, p.torus_bits, np.arange(4), base=p.torus_base)
    d_lut = torch.from_numpy(lut).cuda()
    out = api.functional_bootstrapping_mp_ntt(ctx, key, lwe, d_lut)
    out2 = api.functional_bootstrapping_mp_ntt(ctx, key2, lwe, d_lut)
    np.testing.assert_array_equal(out.cpu().numpy(), out2.cpu().numpy())
    np.testing.assert_array_equal(out.cpu().numpy(), ora.pbs(lwe.cpu().numpy(), lut))


@pytest.mark.parametrize("base,n", [(T32_N1024, 630), (T56_N2048, 750)])
def test_gpu_key_and_gpu_encryption_bootstrap_correctly(base, n, built_lib):
    """Full parameter sets: messages in [0, base/2) encrypted on the GPU under a GPU-made key
    come back from the bootstrap with the identity table and decrypt to themselves."""
    from yatfhe_gb300 import api

    p = small(base, n)
    ctx = api.Context(p, 0)
    key, lwe_s, rlwe_s = api.keygen(ctx, 11, p.lwe_noise_b, p.rlwe_noise_b, return_secrets=True)
    half = p.torus_base // 2
    msgs = np.arange(512) % half
    mu = msgs.astype(np.int64) << (32 - int(np.log2(p.torus_base)))
    lwe = api.sym_enc_tlwe(ctx, torch.from_numpy(lwe_s).cuda(), torch.from_numpy(mu).cuda(), 99, 1, p.lwe_noise_b)
    ora = Restatement(p)
    ora.set_keys(lwe_s, rlwe_s)
    np.testing.assert_array_equal(ora.decrypt(lwe.cpu().numpy(), p.torus_base), msgs)
    lut = lutmod.padded_message_lut(p.N, p.torus_bits, np.arange(half), base=p.torus_base)
    out = api.functional_bootstrapping_mp_ntt(ctx, key, lwe, torch.from_numpy(lut).cuda())
    np.testing.assert_array_equal(ora.decrypt(out.cpu().numpy(), p.torus_base), msgs)


def test_draws_are_deterministic_and_distributed(built_lib):
    from yatfhe_gb300 import api

    p = small(T32_N1024, 64)
    ctx = api.Context(p, 0)
    b = 3
    a = api.draw_keygen_samples(ctx, 1234, b, b)
    again = api.draw_keygen_samples(ctx, 1234, b, b)
    other = api.draw_keygen_samples(ctx, 1235, b, b)
    for f in a:
        np.testing.assert_array_equal(a[f], again[f])
        assert not np.array_equal(a[f], other[f]), f
    # binary secrets, about half ones
    for f in ("lwe_s", "rlwe_s"):
        assert set(np.unique(a[f])) <= {0, 1}
        assert abs(a[f].mean() - 0.5) < 0.12
    # TUniform(b): values -2^b .. 2^b, the two ends with probability 2^-(b+2), the rest 2^-(b+1)
    noise = a["bsk_noise"].ravel().astype(np.int64)
    counts = np.bincount(noise + (1 << b), minlength=(2 << b) + 1)
    assert counts.size == (2 << b) + 1
    prob = np.full((2 << b) + 1, 2.0 ** -(b + 1))
    prob[0] = prob[-1] = 2.0 ** -(b + 2)
    expect = prob * noise.size
    chi2 = float(((counts - expect) ** 2 / expect).sum())
    assert chi2 < 40.0, (chi2, counts)  # 16 degrees of freedom: p ~ 1e-3 at 39.3
    kn = a["ksk_noise"].ravel()
    assert kn.min() >= -(1 << b) and kn.max() <= 1 << b
    # masks mod q: below q, uniform (mean q / 2, every top bucket hit)
    m = a["bsk_mask"].ravel()
    q = Restatement(p).q
    assert int(m.max()) < q
    assert abs(float(m.mean()) / q - 0.5) < 0.01
    buckets = np.bincount((m // np.uint64(q // 16 + 1)).astype(np.int64), minlength=16)
    assert buckets.min() > m.size / 16 * 0.95, buckets
    # uniform 32-bit KSK masks: each bit set half the time
    km = a["ksk_mask"].ravel().view(np.uint32)
    bits = ((km[:, None] >> np.arange(32, dtype=np.uint32)) & 1).mean(axis=0)
    assert np.all(np.abs(bits - 0.5) < 0.01), bits


def test_encrypt_draws_depend_on_seed_and_call(built_lib):
    from yatfhe_gb300 import api

    p = small(T32_N1024, 630)
    ctx = api.Context(p, 0)
    s = torch.from_numpy((np.arange(p.n) % 3 == 0).astype(np.int32)).cuda()
    mu = torch.zeros(4000, dtype=torch.int64, device="cuda")
    x = api.sym_enc_tlwe(ctx, s, mu, 5, 0, 4).cpu().numpy()
    np.testing.assert_array_equal(x, api.sym_enc_tlwe(ctx, s, mu, 5, 0, 4).cpu().numpy())
    y = api.sym_enc_tlwe(ctx, s, mu, 5, 1, 4).cpu().numpy()
    z = api.sym_enc_tlwe(ctx, s, mu, 6, 0, 4).cpu().numpy()
    assert (x[:, :p.n] != y[:, :p.n]).mean() > 0.99 and (x[:, :p.n] != z[:, :p.n]).mean() > 0.99
    # b - <a, s> is the noise: TUniform(4), |e| <= 16, mean about 0
    a = x[:, :p.n].astype(np.int64)
    e = ((x[:, p.n].astype(np.int64) - (a * s.cpu().numpy()).sum(axis=1)) % (1 << 32))
    e = np.where(e >= 1 << 31, e - (1 << 32), e)
    assert np.abs(e).max() <= 16 and abs(e.mean()) < 1.0  # standard error of the mean ~0.15
    # every ciphertext's mask differs from every other's
    assert len({r.tobytes() for r in x[:, :p.n]}) == len(x)


@pytest.mark.parametrize("base", [T32_N1024, T56_N2048])
def test_rlwe_encrypt_from_samples_matches_restatement(base, built_lib):
    """symEncTrlweMultiSampleSimple fed the restatement's draws: bit-exact NTT-domain samples;
    an unreduced mask word is refused."""
    from yatfhe_gb300 import api

    p = small(base, 8)
    ora = Restatement(p)
    ora.keygen(9)
    _, rlwe_s = ora.keys()
    rng = np.random.default_rng(6)
    half = 1 << (p.torus_bits - 1)
    mu = rng.integers(-half, half, (5, p.N), dtype=np.int64)
    want, mask, noise = ora.encrypt_rlwe_ntt_samples(mu)
    ctx = api.Context(p, 0)
    d_s = torch.from_numpy(rlwe_s).cuda()
    d_mu = torch.from_numpy(mu).cuda()
    got = api.sym_enc_trlwe_ntt_from_samples(ctx, d_s, d_mu, torch.from_numpy(mask.view(np.int64)).cuda(),
                                             torch.from_numpy(noise).cuda())
    np.testing.assert_array_equal(got.cpu().numpy().view(np.uint64), want)
    bad = mask.copy()
    bad[3, 0, 17] = np.uint64(ora.q)
    with pytest.raises(Exception, match="not reduced"):
        api.sym_enc_trlwe_ntt_from_samples(ctx, d_s, d_mu, torch.from_numpy(bad.view(np.int64)).cuda(),
                                           torch.from_numpy(noise).cuda())


@pytest.mark.parametrize("base", [T32_N1024, T56_N2048])
def test_rlwe_encrypt_drawn_decrypts(base, built_lib):
    """GPU-drawn RLWE encryptions: INTT(b - a . NTT(s)) is mu plus TUniform(rlwe_noise_b) noise,
    the masks are reduced, and (seed, call) fixes the samples."""
    from yatfhe_gb300 import api

    p = small(base, 8)
    ora = Restatement(p)
    q = ora.q
    rng = np.random.default_rng(8)
    rlwe_s = rng.integers(0, 2, p.k * p.N).astype(np.int32)
    half = 1 << (p.torus_bits - 1)
    mu = rng.integers(-half, half, (3, p.N), dtype=np.int64)
    ctx = api.Context(p, 0)
    d_s = torch.from_numpy(rlwe_s).cuda()
    d_mu = torch.from_numpy(mu).cuda()
    out = api.sym_enc_trlwe_ntt(ctx, d_s, d_mu, 21, 4, p.rlwe_noise_b).cpu().numpy().view(np.uint64)
    again = api.sym_enc_trlwe_ntt(ctx, d_s, d_mu, 21, 4, p.rlwe_noise_b).cpu().numpy().view(np.uint64)
    other = api.sym_enc_trlwe_ntt(ctx, d_s, d_mu, 21, 5, p.rlwe_noise_b).cpu().numpy().view(np.uint64)
    np.testing.assert_array_equal(out, again)
    assert (out[:, 0] != other[:, 0]).mean() > 0.99
    assert int(out.max()) < q
    s_ntt = [int(x) for x in ora.ntt_forward(rlwe_s.astype(np.int64))]
    bound = 1 << p.rlwe_noise_b
    for i in range(len(mu)):
        a = [int(x) for x in out[i, 0]]
        b = [int(x) for x in out[i, 1]]
        diff = np.array([(bj - aj * sj) % q for aj, bj, sj in zip(a, b, s_ntt)], np.uint64)
        phase = ora.ntt_inverse(diff)
        e = (phase - mu[i]) & ((1 << p.torus_bits) - 1)
        e = np.where(e >= half, e - (1 << p.torus_bits), e)
        assert np.abs(e).max() <= bound and np.abs(e).max() > bound // 4, (i, np.abs(e).max())


def test_sampling_arguments(built_lib):
    """Empty batches are no-ops; out-of-range noise widths and unreduced masks are refused."""
    from yatfhe_gb300 import api

    p = small(T32_N1024, 16)
    ctx = api.Context(p, 0)
    s = torch.zeros(p.n, dtype=torch.int32, device="cuda")
    mu = torch.zeros(0, dtype=torch.int64, device="cuda")
    assert api.sym_enc_tlwe(ctx, s, mu, 1, 0, 4).shape == (0, p.n + 1)
    rs = torch.zeros(p.N, dtype=torch.int32, device="cuda")
    rmu = torch.zeros((0, p.N), dtype=torch.int64, device="cuda")
    assert api.sym_enc_trlwe_ntt(ctx, rs, rmu, 1, 0, 4).shape == (0, 2, p.N)
    with pytest.raises(Exception):
        api.sym_enc_tlwe(ctx, s, torch.zeros(4, dtype=torch.int64, device="cuda"), 1, 0, 31)
    with pytest.raises(Exception):
        api.keygen(ctx, 1, 18, 31)
    with pytest.raises(Exception):
        api.draw_keygen_samples(ctx, 1, -1, 8)

"""GPU parity: the CUDA bootstrap against the oracle, bit for bit, through the C ABI.

Keys come from the oracle's seeded key generation (bit-identical to the reference's own,
checked on CPU in test_oracle.py); the GPU path receives them exactly as a reference user
would hand them over (NTT-domain key words / the reference's key file format).
"""
import numpy as np
import pytest

from oracle.oracle import Restatement
from yatfhe_gb300 import lut as lutmod
from yatfhe_gb300.params import T32_N1024, T56_N2048, small

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _sign_inputs(ora, count, seed):
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 2, count)
    mu = np.where(bits == 1, 1 << 29, -(1 << 29)).astype(np.int64)
    return mu, ora.encrypt(mu)


def _setup(p, seed, built_lib):
    from yatfhe_gb300 import api

    ora = Restatement(p)
    ora.keygen(seed)
    ctx = api.Context(p, 0)
    key = api.BootstrapKey.from_ntt_words(ctx, ora.bsk_ntt()).set_ksk(ora.ksk())
    return ora, ctx, key


@pytest.fixture(scope="module")
def t32_small(built_lib):
    return _setup(small(T32_N1024, 32), 0x5EED0001, built_lib)


@pytest.fixture(scope="module")
def t56_small(built_lib):
    return _setup(small(T56_N2048, 12), 0x5EED0003, built_lib)


def _pbs_gpu(ctx, key, lwe, lut):
    from yatfhe_gb300 import api

    out = api.functional_bootstrapping_mp_ntt(ctx, key, torch.from_numpy(lwe).cuda(), torch.from_numpy(lut).cuda())
    return out.cpu().numpy()


def test_pbs_t32_small_bit_exact(t32_small):
    ora, ctx, key = t32_small
    mu, lwe = _sign_inputs(ora, 16, 1)
    lut = lutmod.sign_lut(ctx.params.N, 32)
    got = _pbs_gpu(ctx, key, lwe, lut)
    np.testing.assert_array_equal(got, ora.pbs(lwe, lut, threads=8))
    np.testing.assert_array_equal(ora.decrypt(got, 8), np.where(mu > 0, 1, -1))


@pytest.mark.parametrize("layout", [0, 2])
def test_blind_rotate_checkpoints_t32(t32_small, layout):
    """Accumulator after 1, 2, 7 and all CMux steps equals the oracle's trace (channel and
    row-cluster layouts)."""
    from yatfhe_gb300 import api

    ora, ctx, key = t32_small
    api.set_launch(ctx, 1, 0, layout)
    _, lwe = _sign_inputs(ora, 2, 2)
    lut = ora.test_polynomial(0, 8)
    cps = [0, 1, 6, ctx.params.n - 1]
    d_in = torch.from_numpy(lwe).cuda()
    d_lut = torch.from_numpy(lut).cuda()
    for c in range(len(lwe)):
        want, final = ora.blind_rotate_trace(lwe[c], lut, cps)
        for k, step in enumerate(cps):
            acc = api.blind_rotate_mp21_ntt(ctx, key, d_in[c:c + 1], d_lut, steps=step + 1).cpu().numpy()[0]
            np.testing.assert_array_equal(acc, want[k], err_msg=f"ciphertext {c}, after step {step}")
        np.testing.assert_array_equal(want[-1], final)
    api.set_launch(ctx, 1, 0, 0)


@pytest.mark.parametrize("layout", [0, 2])
def test_blind_rotate_acc_reference_semantics(t32_small, layout):
    """yg_blind_rotate_acc = blindRotateMP21Ntt(accum, bsk, scaled, param): a caller-built
    accumulator and already-switched mask, rotated in place (channel and row-cluster
    layouts)."""
    import ctypes

    from yatfhe_gb300 import _lib, api

    ora, ctx, key = t32_small
    api.set_launch(ctx, 1, 0, layout)
    p = ctx.params
    _, lwe = _sign_inputs(ora, 3, 8)
    lut = ora.test_polynomial(1, 8)
    scaled = np.stack([ora.modswitch(c) for c in lwe])
    acc0 = np.zeros((3, 2 * p.N), np.int64)
    for c in range(3):
        acc0[c, p.N:] = ora.rotate(lut, -int(scaled[c, p.n]), False)
    d_a = torch.from_numpy(np.ascontiguousarray(scaled[:, :p.n])).cuda()
    d_acc = torch.from_numpy(acc0).cuda()
    _lib.check(_lib.lib().yg_blind_rotate_acc(ctx.handle, key.handle, ctypes.c_void_p(d_a.data_ptr()),
                                              ctypes.c_void_p(d_acc.data_ptr()), 3, ctypes.c_void_p(0)))
    got = d_acc.cpu().numpy()
    for c in range(3):
        _, final = ora.blind_rotate_trace(lwe[c], lut, [])
        np.testing.assert_array_equal(got[c], final)
    api.set_launch(ctx, 1, 0, 0)


@pytest.mark.parametrize("layout", [2, 3])
@pytest.mark.parametrize("levels", [3, 4])
def test_cluster_key_stage_with_skipped_steps(levels, layout, built_lib):
    """The cluster layouts copy each active step's key rows into shared memory by TMA (the
    row cluster for l <= 3, reading them from global memory at l = 4; the channel cluster at
    every l): with CMux steps skipped (a_i = 0) at the start, in the middle and at the end,
    40 ciphertexts give the oracle's bootstrap, no bounded wait gave up, and the result
    equals the channel layout's."""
    import ctypes
    import dataclasses

    from yatfhe_gb300 import _lib, api

    p = dataclasses.replace(small(T32_N1024, 24), l=levels, l_approx=levels, radix_bits=7 if levels == 3 else 5)
    ora, ctx, key = _setup(p, 0x5EED0011 + levels, built_lib)
    mu, lwe = _sign_inputs(ora, 40, 30 + levels)
    for c in range(0, 40, 2):  # even ciphertexts: a few mask words 0, so those steps are skipped
        lwe[c, [0, 1, 7, p.n - 1]] = 0
    lut = lutmod.sign_lut(p.N, 32)
    api.set_launch(ctx, 1, 0, 0)
    want = _pbs_gpu(ctx, key, lwe, lut)
    api.set_launch(ctx, 1, 0, layout)
    got = _pbs_gpu(ctx, key, lwe, lut)
    api.set_launch(ctx, 1, 0, 0)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(got[:6], ora.pbs(lwe[:6], lut, threads=8))
    n = ctypes.c_uint64(99)
    _lib.check(_lib.lib().yg_wait_timeouts(ctx.handle, ctypes.byref(n)))
    assert n.value == 0


def test_keyswitch_alone_t32(t32_small):
    from yatfhe_gb300 import api

    ora, ctx, key = t32_small
    p = ctx.params
    rng = np.random.default_rng(3)
    big = rng.integers(-(1 << 31), 1 << 31, size=(5, p.k * p.N + 1), dtype=np.int64).astype(np.int32)
    big[0, :] = np.int32(-(1 << 31))  # extreme words
    big[1, :] = 0
    got = api.switch_key_for_tlwe(ctx, key, torch.from_numpy(big).cuda()).cpu().numpy()
    for c in range(len(big)):
        np.testing.assert_array_equal(got[c], ora.keyswitch(big[c]))


def test_keyswitch_split_matches_unsplit(t32_small):
    """Small batches split the input coefficients across CTAs that add into the output; a
    batch large enough to fill the GPU runs unsplit in tiles of 8 ciphertexts, a larger one
    in tiles of 32.  A ciphertext's key switch is the same in batches of 1, 3, 9, 61, 6,000
    and 20,000 (extreme words included), and equals the oracle's."""
    from yatfhe_gb300 import api

    ora, ctx, key = t32_small
    p = ctx.params
    rng = np.random.default_rng(31)
    big = rng.integers(-(1 << 31), 1 << 31, size=(20000, p.k * p.N + 1), dtype=np.int64).astype(np.int32)
    big[0, :] = np.int32(-(1 << 31))
    big[1, :] = np.int32((1 << 31) - 1)
    d_big = torch.from_numpy(big).cuda()
    full = api.switch_key_for_tlwe(ctx, key, d_big).cpu().numpy()
    for count in (1, 3, 9, 61, 6000):
        got = api.switch_key_for_tlwe(ctx, key, d_big[:count].contiguous()).cpu().numpy()
        np.testing.assert_array_equal(got, full[:count], err_msg=f"batch of {count}")
    for c in (0, 1, 2, 5999, 19999):
        np.testing.assert_array_equal(full[c], ora.keyswitch(big[c]))


def test_pbs_t56_small_bit_exact(t56_small):
    ora, ctx, key = t56_small
    rng = np.random.default_rng(4)
    m = rng.integers(0, 16, 12)
    table = rng.integers(0, 16, 16)
    mu = (m * (1 << 27)).astype(np.int64)  # m 2^32 / 32
    lwe = ora.encrypt(mu)
    lut = lutmod.padded_message_lut(ctx.params.N, 56, table)
    got = _pbs_gpu(ctx, key, lwe, lut)
    np.testing.assert_array_equal(got, ora.pbs(lwe, lut, threads=8))


def test_pbs_empty_and_single(t32_small):
    from yatfhe_gb300 import api

    ora, ctx, key = t32_small
    lut = torch.from_numpy(lutmod.sign_lut(ctx.params.N, 32)).cuda()
    empty = torch.empty((0, ctx.params.n + 1), dtype=torch.int32, device="cuda")
    assert api.functional_bootstrapping_mp_ntt(ctx, key, empty, lut).shape == (0, ctx.params.n + 1)
    _, lwe = _sign_inputs(ora, 1, 5)
    got = _pbs_gpu(ctx, key, lwe, lut.cpu().numpy())
    np.testing.assert_array_equal(got, ora.pbs(lwe, lut.cpu().numpy()))


@pytest.mark.parametrize("which", ["t32", "t56"])
def test_pbs_full_size_bit_exact(which, built_lib):
    """Full parameter sets: n = 630 / N = 1024 with 256 sign-bootstrapped ciphertexts of
    random bits (the CPU-runnable sign bootstrap workload, keyset seed 0x5EED0001), and
    n = 750 / N = 2048 with 4-bit messages through a random lookup table."""
    if which == "t32":
        p, seed = T32_N1024, 0x5EED0001
    else:
        p, seed = T56_N2048, 0x5EED0003
    ora, ctx, key = _setup(p, seed, built_lib)
    rng = np.random.default_rng(6)
    if which == "t32":
        mu, lwe = _sign_inputs(ora, 256, 7)
        lut = lutmod.sign_lut(p.N, 32)
        expect = np.where(mu > 0, 1, -1)
        base = 8
    else:
        m = rng.integers(0, 16, 48)
        table = rng.integers(0, 16, 16)
        lwe = ora.encrypt((m * (1 << 27)).astype(np.int64))
        lut = lutmod.padded_message_lut(p.N, 56, table)
        expect = table[m]
        base = 32
    got = _pbs_gpu(ctx, key, lwe, lut)
    want = ora.pbs(lwe, lut, threads=16)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(ora.decrypt(got, base), expect)


def test_key_words_must_be_reduced(built_lib):
    """A key word >= q is rejected (std::invalid_argument in the reference's NTT loader)."""
    from yatfhe_gb300 import api

    p = small(T32_N1024, 4)
    ctx = api.Context(p, 0)
    words = np.zeros(p.bsk_ntt_words, np.uint64)
    words[123] = p.q_ntt
    with pytest.raises(ValueError):
        api.BootstrapKey.from_ntt_words(ctx, words)
    words[123] = p.q_ntt - 1
    api.BootstrapKey.from_ntt_words(ctx, words).close()


@pytest.mark.parametrize("count", [100, 16384])
def test_pbs_host_buffers(count, built_lib):
    """yg_pbs_host (host buffers in and out; from 16,384 ciphertexts on in four chunks on two
    streams) equals the device-buffer bootstrap and the oracle."""
    from yatfhe_gb300 import api

    p = small(T32_N1024, 8)
    ora, ctx, key = _setup(p, 0x5EED0009, built_lib)
    rng = np.random.default_rng(count)
    lwe = rng.integers(-(1 << 31), 1 << 31, size=(count, p.n + 1), dtype=np.int64).astype(np.int32)
    lut = lutmod.sign_lut(p.N, 32)
    host = api.functional_bootstrapping_mp_ntt_host(ctx, key, lwe, lut)
    dev = _pbs_gpu(ctx, key, lwe, lut)
    np.testing.assert_array_equal(host, dev)
    pick = rng.choice(count, 6, replace=False)
    np.testing.assert_array_equal(host[pick], ora.pbs(lwe[pick], lut))

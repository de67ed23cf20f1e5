"""GPU tests of the group-g key family (group_blind_rotate_kernel: blindRotateNtt, groups 1-3):
bootstrap outputs and accumulators equal to the reference's own (golden fixtures, full size),
equal to the restatement on random ciphertexts and test polynomials, and the entry points
that take GINX rows only refuse the key."""
import hashlib
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import Restatement
from yatfhe_gb300.params import PbsParams, T32_N1024, T56_N2048, small

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def _sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["group2_t32_n1024_seed5eed000c", "group3_t32_n1024_seed5eed000d",
                                  "group1_t32_n1024_seed5eed000e", "group2_t56_n2048_seed5eed000f"])
def test_gpu_reproduces_reference_group_golden(name, built_lib):
    from yatfhe_gb300 import api

    g = np.load(GOLDEN / f"{name}.npz")
    p = PbsParams(*[int(x) for x in g["params"]])
    grp = int(g["group"][0])
    ora = Restatement(p)
    ora.keygen_group(int(g["seed"][0]), grp)
    words = ora.group_words()
    assert _sha(words) == str(g["sha_key"])  # the reference's key
    ctx = api.Context(p, 0)
    key = api.BootstrapKey.from_group_words(ctx, words, grp).set_ksk(ora.ksk())
    d_in = torch.from_numpy(g["lwe_in"]).cuda()
    d_lut = torch.from_numpy(g["lut"]).cuda()
    out = api.functional_bootstrapping_ntt(ctx, key, d_in, d_lut).cpu().numpy()
    np.testing.assert_array_equal(out, g["lwe_out"])
    np.testing.assert_array_equal(ora.decrypt(out, int(g["base"][0])), g["decrypted"])
    acc = api.blind_rotate_ntt(ctx, key, d_in[:1], d_lut).cpu().numpy()[0]
    np.testing.assert_array_equal(acc.reshape(-1), g["acc0"])


@pytest.mark.parametrize("base,group", [(T32_N1024, 1), (T32_N1024, 2), (T32_N1024, 3), (T56_N2048, 2),
                                        (T56_N2048, 3)])
def test_gpu_group_equals_restatement_on_random_inputs(base, group, built_lib):
    """48 random ciphertexts (some with zero masks: skipped and zero rotations) and a random
    test polynomial at n = 12."""
    from yatfhe_gb300 import api

    p = small(base, 12)
    ora = Restatement(p)
    ora.keygen_group(41 + group, group)
    ctx = api.Context(p, 0)
    key = api.BootstrapKey.from_group_words(ctx, ora.group_words(), group).set_ksk(ora.ksk())
    rng = np.random.default_rng(group)
    lwe = rng.integers(-(1 << 31), 1 << 31, size=(48, p.n + 1), dtype=np.int64).astype(np.int32)
    lwe[1, : p.n // 2] = 0
    lwe[2, :] = 0
    lut = rng.integers(-(1 << (p.torus_bits - 1)), 1 << (p.torus_bits - 1), size=p.N, dtype=np.int64)
    d_in, d_lut = torch.from_numpy(lwe).cuda(), torch.from_numpy(lut).cuda()
    acc = api.blind_rotate_ntt(ctx, key, d_in, d_lut).cpu().numpy()
    for c in (0, 1, 2, 47):
        np.testing.assert_array_equal(acc[c], ora.blind_rotate_group(lwe[c], lut), err_msg=f"ciphertext {c}")
    out = api.functional_bootstrapping_ntt(ctx, key, d_in, d_lut).cpu().numpy()
    np.testing.assert_array_equal(out, ora.pbs_group(lwe, lut, threads=8))
    host = api.functional_bootstrapping_mp_ntt_host(ctx, key, lwe, lut)
    np.testing.assert_array_equal(host, out)


def test_gpu_group_refusals(built_lib):
    from yatfhe_gb300 import api

    p = small(T32_N1024, 6)
    ora = Restatement(p)
    ora.keygen_group(5, 2)
    ctx = api.Context(p, 0)
    key = api.BootstrapKey.from_group_words(ctx, ora.group_words(), 2).set_ksk(ora.ksk())
    lut = torch.zeros(p.N, dtype=torch.int64, device="cuda")
    d_in = torch.zeros((4, p.n + 1), dtype=torch.int32, device="cuda")
    with pytest.raises(ValueError, match="keys run through"):
        api.BatchPlan(ctx, [key], [lut], 4)
    with pytest.raises(ValueError, match="steps = n"):
        api.blind_rotate_mp21_ntt(ctx, key, d_in, lut, steps=2)
    w = ora.group_words().copy()
    w[0, 0, 0, 0, 0] = ora.q  # not reduced mod q
    with pytest.raises(ValueError, match="not reduced"):
        api.BootstrapKey.from_group_words(ctx, w, 2)
    import ctypes

    from yatfhe_gb300 import _lib

    ok = np.ascontiguousarray(ora.group_words())
    h = ctypes.c_void_p()
    with pytest.raises(ValueError, match="group 1, 2 or 3"):
        _lib.check(_lib.lib().yg_key_upload_group(ctx.handle, ctypes.c_void_p(ok.ctypes.data), 4, p.l, ctypes.byref(h)))


def test_gpu_group_rotates_a_given_accumulator(built_lib):
    """yg_blind_rotate_acc with a group key (the adapter's blindRotateNtt): the mask already
    switched to mod 2N and the accumulator after genNoiselessTrlweSample, rotated in place,
    equal to the restatement's blind rotation."""
    import ctypes

    from yatfhe_gb300 import _lib, api

    p = small(T32_N1024, 12)
    ora = Restatement(p)
    ora.keygen_group(17, 2)
    ctx = api.Context(p, 0)
    key = api.BootstrapKey.from_group_words(ctx, ora.group_words(), 2)
    rng = np.random.default_rng(11)
    lwe = rng.integers(-(1 << 31), 1 << 31, size=(6, p.n + 1), dtype=np.int64).astype(np.int32)
    lut = rng.integers(-(1 << 31), 1 << 31, size=p.N, dtype=np.int64)
    scaled = np.stack([ora.modswitch(x) for x in lwe])
    acc = np.zeros((len(lwe), 2 * p.N), np.int64)
    for c in range(len(lwe)):
        acc[c, p.N:] = ora.rotate(lut, -int(scaled[c, p.n]), False)  # genNoiselessTrlweSample
    d_scaled = torch.from_numpy(np.ascontiguousarray(scaled[:, : p.n])).cuda()
    d_acc = torch.from_numpy(acc).cuda()
    _lib.check(_lib.lib().yg_blind_rotate_acc(ctx.handle, key.handle, ctypes.c_void_p(d_scaled.data_ptr()),
                                              ctypes.c_void_p(d_acc.data_ptr()), len(lwe), None))
    got = d_acc.cpu().numpy()
    for c in range(len(lwe)):
        np.testing.assert_array_equal(got[c], ora.blind_rotate_group(lwe[c], lut), err_msg=f"ciphertext {c}")

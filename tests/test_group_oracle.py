"""CPU tests of the group-g key family of blindRotateNtt (BootstrappingKey with TrgswDft rows;
group 1: blindRotateNormalNtt, groups 2 and 3: blindRotateGroup2Ntt / blindRotateGroup3Ntt,
yatfhe/src/blind_rotate.cpp:202-560) in the oracle: the plain-C restatement of its key
generation (genBootstrappingKey, yatfhe/src/bootstrapping.cpp:16-38,98-104) and of
functionalBootstrappingNtt (:60-68), against the golden fixtures made by the reference's own
code (tests/golden/make_golden.py) and, where the reference tree is present, against the
reference itself."""
import hashlib
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as o
from oracle.oracle import Restatement
from yatfhe_gb300 import lut as lutmod
from yatfhe_gb300.params import PbsParams, T32_N1024, T56_N2048, WWL24_T32_N2048, small

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ["group2_t32_n1024_seed5eed000c", "group3_t32_n1024_seed5eed000d", "group1_t32_n1024_seed5eed000e",
         "group2_t56_n2048_seed5eed000f"]
needs_reference = pytest.mark.skipif(not o.reference_available(), reason="reference tree not present")


def _sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", CASES)
def test_restatement_reproduces_reference_group_golden(name):
    g = np.load(GOLDEN / f"{name}.npz")
    p = PbsParams(*[int(x) for x in g["params"]])
    grp = int(g["group"][0])
    ora = Restatement(p)
    ora.keygen_group(int(g["seed"][0]), grp)
    s, z = ora.keys()
    assert _sha(s) == str(g["sha_lwe_s"]) and _sha(z) == str(g["sha_rlwe_s"])
    assert _sha(ora.group_words()) == str(g["sha_key"])
    assert _sha(ora.ksk()) == str(g["sha_ksk"])
    np.testing.assert_array_equal(ora.blind_rotate_group(g["lwe_in"][0], g["lut"]), g["acc0"])
    out = ora.pbs_group(g["lwe_in"], g["lut"], threads=8)
    np.testing.assert_array_equal(out, g["lwe_out"])
    np.testing.assert_array_equal(ora.decrypt(out, int(g["base"][0])), g["decrypted"])


def test_group_keys_encrypt_the_indicator_patterns():
    """TRGSW k2 of a group encrypts [combined == k2] (the reference's GROUP2_KEYGEN test,
    google_tests/bootstrappping_test.cpp:33-83): the b row of level 0 minus a . s is
    mu 2^(T - radix) plus small noise."""
    p = small(T32_N1024, 6)
    ora = Restatement(p)
    ora.keygen_group(3, 3)
    s, z = ora.keys()
    w = ora.group_words()
    zz = z.astype(np.int64)
    for blk in range(2):
        combined = sum(int(s[blk * 3 + i2]) << (2 - i2) for i2 in range(3))
        for k2 in range(8):
            a = ora.ntt_inverse(w[blk * 8 + k2, 0, 1, 0])
            b = ora.ntt_inverse(w[blk * 8 + k2, 0, 1, 1])
            # b - a s (negacyclic), coefficient 0, on the 32-bit torus
            as0 = int(a[0] * zz[0] - np.dot(a[1:], zz[::-1][:-1]))
            phase = (int(b[0]) - as0) % (1 << 32)
            phase = phase - (1 << 32) if phase >= 1 << 31 else phase
            mu = round(phase / (1 << (32 - p.radix_bits)))
            assert mu == (1 if combined == k2 else 0), (blk, k2, phase)


def test_group_must_divide_n():
    ora = Restatement(small(T32_N1024, 7))
    with pytest.raises(RuntimeError, match="divide n"):
        ora.keygen_group(1, 2)


@needs_reference
@pytest.mark.parametrize("base,group", [(T32_N1024, 1), (T32_N1024, 2), (T32_N1024, 3), (T56_N2048, 2),
                                        (WWL24_T32_N2048, 3)])
def test_group_matches_reference(base, group):
    """Small-n keys, accumulators and outputs against the reference's own code."""
    p = small(base, 6)
    ref, ora = o.Reference(p), Restatement(p)
    ref.keygen_group(21, group)
    ora.keygen_group(21, group)
    np.testing.assert_array_equal(ref.group_words(), ora.group_words())
    np.testing.assert_array_equal(ref.ksk(), ora.ksk())
    rng = np.random.default_rng(5)
    mu = np.where(rng.integers(0, 2, 3) == 1, 1 << 29, -(1 << 29)).astype(np.int64)
    lwe = ref.encrypt(mu)
    v = lutmod.sign_lut(p.N, p.torus_bits)
    out, acc0 = ref.pbs_group(lwe, v, with_acc=True)
    np.testing.assert_array_equal(ora.blind_rotate_group(lwe[0], v), acc0)
    np.testing.assert_array_equal(ora.pbs_group(lwe, v, threads=3), out)

"""CPU tests of the lazy ("OURS") key family in the oracle: the plain-C restatement of its key
generation (genBootstrappingKeyMPLazyPipeAlt, yatfhe/src/bootstrapping.cpp:322-339), of its
blind rotation (blindRotateLazyPipeAltNtt, yatfhe/src/blind_rotate.cpp:995-1135) and of its
file format (serializeBskLazyPipeAlt, yatfhe/src/ya_serializer.cpp:445-481), against the golden
fixtures made by the reference's own code (tests/golden/make_golden.py) and, where the
reference tree is present, against the reference itself."""
import hashlib
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as o
from oracle.oracle import Restatement
from yatfhe_gb300 import lut as lutmod
from yatfhe_gb300.params import PbsParams, WWL24_T32_N2048, WWL24_T56_N2048, small

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ["lazy_t32_n2048_seed5eed0007", "lazy_t56_n2048_seed5eed0008"]
needs_reference = pytest.mark.skipif(not o.reference_available(), reason="reference tree not present")


def _sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _golden(name):
    g = np.load(GOLDEN / f"{name}.npz")
    return g, PbsParams(*[int(x) for x in g["params"]])


@pytest.mark.parametrize("name", CASES)
def test_restatement_reproduces_reference_lazy_golden(name):
    """Keys from the recorded seed, the accumulator of ciphertext 0 after the lazy blind
    rotation, and the bootstrap outputs equal the reference's."""
    g, p = _golden(name)
    ora = Restatement(p)
    ora.keygen_lazy(int(g["seed"][0]))
    s, z = ora.keys()
    cprime, s2 = ora.lazy_words()
    assert _sha(s) == str(g["sha_lwe_s"]) and _sha(z) == str(g["sha_rlwe_s"])
    assert _sha(cprime) == str(g["sha_cprime"]) and _sha(s2) == str(g["sha_s2"])
    assert _sha(ora.ksk()) == str(g["sha_ksk"])
    np.testing.assert_array_equal(ora.blind_rotate_lazy(g["lwe_in"][0], g["lut"]), g["acc0"])
    out = ora.pbs_lazy(g["lwe_in"], g["lut"], threads=8)
    np.testing.assert_array_equal(out, g["lwe_out"])
    np.testing.assert_array_equal(ora.decrypt(out, int(g["base"][0])), g["decrypted"])


def test_lazy_key_is_the_wwl24_key_in_the_coefficient_domain():
    """The two families draw the same samples: the lazy rows are the WWL+24 rows taken back to
    the torus, the s2 keys are equal."""
    p = small(WWL24_T32_N2048, 4)
    a, b = Restatement(p), Restatement(p)
    a.keygen_lazy(9)
    b.keygen_wwl24(9)
    cp_lazy, s2_lazy = a.lazy_words()
    cp_wwl, s2_wwl = b.wwl24_words()
    np.testing.assert_array_equal(s2_lazy, s2_wwl)
    for i, lvl, poly in [(0, 0, 0), (3, 3, 1), (2, 1, 1)]:
        np.testing.assert_array_equal(b.ntt_inverse(cp_wwl[i, lvl, poly]), cp_lazy[i, lvl, poly])


def test_lazy_file_round_trip(tmp_path):
    p = small(WWL24_T32_N2048, 5)
    a = Restatement(p)
    a.keygen_lazy(3)
    a.save_lazy_file(tmp_path / "k.bin")
    b = Restatement(p)
    b.load_lazy_file(tmp_path / "k.bin")
    for x, y in zip(a.lazy_words(), b.lazy_words()):
        np.testing.assert_array_equal(x, y)
    # s2 (8 + l TrlweDft) + n half TrgswMP (13 + L Trlwe of int32 words) + 8 bytes
    trlwe_dft = 4 + 1 + (4 + 8 * p.N) + 4 + (4 + 8 * p.N)
    trlwe = 4 + 4 + (4 + 4 * p.N) + 4 + (4 + 4 * p.N)
    assert (tmp_path / "k.bin").stat().st_size == 8 + p.l * trlwe_dft + p.n * (13 + p.l_approx * trlwe) + 8
    raw = (tmp_path / "k.bin").read_bytes()
    (tmp_path / "short.bin").write_bytes(raw[:-100])
    with pytest.raises(RuntimeError, match="not a lazy key"):
        b.load_lazy_file(tmp_path / "short.bin")


def test_lazy_needs_two_key_components():
    p = small(WWL24_T32_N2048, 1)
    a = Restatement(p)
    a.keygen_lazy(1)
    with pytest.raises(RuntimeError, match="n < 2"):
        a.blind_rotate_lazy(np.zeros(p.n + 1, np.int32), lutmod.sign_lut(p.N, 32))


@needs_reference
@pytest.mark.parametrize("base", [WWL24_T32_N2048, WWL24_T56_N2048])
def test_lazy_matches_reference(base, tmp_path):
    """Small-n keys, file interchange in both directions, accumulators and outputs against the
    reference's own code."""
    p = small(base, 6)
    ref, ora = o.Reference(p), Restatement(p)
    ref.keygen_lazy(21)
    ora.keygen_lazy(21)
    for x, y in zip(ref.lazy_words(), ora.lazy_words()):
        np.testing.assert_array_equal(x, y)
    ref.save_lazy_file(tmp_path / "ref.bin")
    ora2 = Restatement(p)
    ora2.load_lazy_file(tmp_path / "ref.bin")
    for x, y in zip(ref.lazy_words(), ora2.lazy_words()):
        np.testing.assert_array_equal(x, y)
    ora.save_lazy_file(tmp_path / "ora.bin")
    assert (tmp_path / "ora.bin").read_bytes() == (tmp_path / "ref.bin").read_bytes()
    rng = np.random.default_rng(5)
    mu = np.where(rng.integers(0, 2, 3) == 1, 1 << 29, -(1 << 29)).astype(np.int64)
    lwe = ref.encrypt(mu)
    v = lutmod.sign_lut(p.N, p.torus_bits)
    out, acc0 = ref.pbs_lazy(lwe, v, with_acc=True)
    np.testing.assert_array_equal(ora.blind_rotate_lazy(lwe[0], v), acc0)
    np.testing.assert_array_equal(ora.pbs_lazy(lwe, v, threads=3), out)


@needs_reference
def test_lazy_sweep_split_gives_the_same_outputs():
    """blindRotateLazyPipeAltNttSweep only splits the pipeline's work differently (how many
    digit levels stageA transforms, how many workers run it): every split gives the outputs
    of blindRotateLazyPipeAltNtt, which is what the adapter maps it to."""
    p = small(WWL24_T32_N2048, 6)
    ref = o.Reference(p)
    ref.keygen_lazy(12)
    rng = np.random.default_rng(3)
    mu = np.where(rng.integers(0, 2, 2) == 1, 1 << 29, -(1 << 29)).astype(np.int64)
    lwe = ref.encrypt(mu)
    v = lutmod.sign_lut(p.N, p.torus_bits)
    want = ref.pbs_lazy(lwe, v)
    for move, units in [(0, 1), (1, 2), (2, 2), (4, 3), (8, 4)]:
        np.testing.assert_array_equal(ref.pbs_lazy_sweep(lwe, v, move, units), want, err_msg=f"{move}, {units}")


@needs_reference
@pytest.mark.parametrize("base", [WWL24_T32_N2048, WWL24_T56_N2048])
def test_lazy_no_first_matches_reference(base):
    """blindRotateLazyPipeAltNoFirstNtt (yatfhe/src/blind_rotate.cpp:1137-1267): the accumulator
    X^-b (0, v) and the ordinary chain for every key index, the first one included.  The
    restatement's accumulators and outputs equal the reference's, with skipped steps (a_0 = 0,
    a run of zeros) among the inputs.  They also equal blindRotateLazyPipeAltNtt's bit for
    bit: the first-component shortcut X^-b ((X^a_0 - 1) derived + (0, v)) is the in-place
    external product of X^-b (0, v) with the first key index's TRGSW, the same exact
    polynomial mod q before the one rounding, so the GPU lazy rotation serves both."""
    p = small(base, 6)
    ref, ora = o.Reference(p), Restatement(p)
    ref.keygen_lazy(23)
    ora.keygen_lazy(23)
    rng = np.random.default_rng(7)
    mu = np.where(rng.integers(0, 2, 4) == 1, 1 << 29, -(1 << 29)).astype(np.int64)
    lwe = ref.encrypt(mu)
    lwe[1, 0] = 0                # a_0 = 0: the first step is skipped
    lwe[2, 1:4] = 0              # a run of skipped steps
    v = lutmod.sign_lut(p.N, p.torus_bits)
    out, acc0 = ref.pbs_lazy(lwe, v, with_acc=True, no_first=True)
    np.testing.assert_array_equal(ora.blind_rotate_lazy(lwe[0], v, no_first=True), acc0)
    np.testing.assert_array_equal(ora.pbs_lazy(lwe, v, threads=3, no_first=True), out)
    np.testing.assert_array_equal(ref.decrypt(out[[0, 3]], 8), np.where(mu[[0, 3]] > 0, 1, -1))
    for c in range(len(lwe)):
        out1, acc1 = ref.pbs_lazy(lwe[c:c + 1], v, with_acc=True)
        out2, acc2 = ref.pbs_lazy(lwe[c:c + 1], v, with_acc=True, no_first=True)
        np.testing.assert_array_equal(acc1, acc2, err_msg=f"accumulator of ciphertext {c}")
        np.testing.assert_array_equal(out1, out2)

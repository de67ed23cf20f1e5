"""CPU tests of the WWL+24 key family in the oracle: the plain-C restatement of its key
generation, of the GINX rows its blind rotation derives (switchTrlweToSecretEmbeddingNtt,
yatfhe/src/trgsw.cpp:861-905) and of its file format, against the golden fixtures made by the
reference's own code (tests/golden/make_golden.py) and, where the reference tree is present,
against the reference itself."""
import hashlib
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as o
from oracle.oracle import Restatement
from yatfhe_gb300 import lut as lutmod
from yatfhe_gb300.params import PbsParams, WWL24_T32_N2048, WWL24_T56_N2048, small

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ["wwl24_t32_n2048_seed5eed0005", "wwl24_t56_n2048_seed5eed0006"]
needs_reference = pytest.mark.skipif(not o.reference_available(), reason="reference tree not present")


def _sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _golden(name):
    g = np.load(GOLDEN / f"{name}.npz")
    return g, PbsParams(*[int(x) for x in g["params"]])


@pytest.mark.parametrize("name", CASES)
def test_restatement_reproduces_reference_wwl24_golden(name):
    """Keys from the recorded seed, the derived GINX rows, and the bootstrap outputs equal the
    reference's (blindRotateWWL24Ntt inside functionalBootstrappingMPNtt's composition)."""
    g, p = _golden(name)
    ora = Restatement(p)
    ora.keygen_wwl24(int(g["seed"][0]))
    s, z = ora.keys()
    cprime, s2 = ora.wwl24_words()
    assert _sha(s) == str(g["sha_lwe_s"]) and _sha(z) == str(g["sha_rlwe_s"])
    assert _sha(cprime) == str(g["sha_cprime"]) and _sha(s2) == str(g["sha_s2"])
    assert _sha(ora.ksk()) == str(g["sha_ksk"])
    assert _sha(ora.wwl24_expanded()) == str(g["sha_expanded"])
    out = ora.pbs(g["lwe_in"], g["lut"], threads=8)  # the GINX bootstrap on the derived rows
    np.testing.assert_array_equal(out, g["lwe_out"])
    np.testing.assert_array_equal(ora.decrypt(out, int(g["base"][0])), g["decrypted"])
    _, acc = ora.blind_rotate_trace(g["lwe_in"][0], g["lut"], [])
    np.testing.assert_array_equal(acc.reshape(-1), g["acc0"])


def test_wwl24_file_round_trip(tmp_path):
    p = small(WWL24_T32_N2048, 5)
    a = Restatement(p)
    a.keygen_wwl24(3)
    a.save_wwl24_file(tmp_path / "k.bin")
    b = Restatement(p)
    b.load_wwl24_file(tmp_path / "k.bin")
    for x, y in zip(a.wwl24_words(), b.wwl24_words()):
        np.testing.assert_array_equal(x, y)
    # n half TRGSW (13 + l TrlweDft) + s2 (8 + l TrlweDft) + 8 bytes
    trlwe = 4 + 1 + (4 + 8 * p.N) + 4 + (4 + 8 * p.N)
    assert (tmp_path / "k.bin").stat().st_size == p.n * (13 + p.l_approx * trlwe) + 8 + p.l * trlwe + 8
    raw = (tmp_path / "k.bin").read_bytes()
    (tmp_path / "short.bin").write_bytes(raw[:-100])
    with pytest.raises(RuntimeError, match="not a WWL"):
        b.load_wwl24_file(tmp_path / "short.bin")


@needs_reference
@pytest.mark.parametrize("base", [WWL24_T32_N2048, WWL24_T56_N2048])
def test_wwl24_matches_reference(base, tmp_path):
    """Small-n keys, derived rows, file interchange in both directions and outputs against the
    reference's own code."""
    p = small(base, 6)
    ref, ora = o.Reference(p), Restatement(p)
    ref.keygen_wwl24(21)
    ora.keygen_wwl24(21)
    for x, y in zip(ref.wwl24_words(), ora.wwl24_words()):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(ref.wwl24_expanded(), ora.wwl24_expanded())
    ref.save_wwl24_file(tmp_path / "ref.bin")
    ora2 = Restatement(p)
    ora2.load_wwl24_file(tmp_path / "ref.bin")
    for x, y in zip(ref.wwl24_words(), ora2.wwl24_words()):
        np.testing.assert_array_equal(x, y)
    ora.save_wwl24_file(tmp_path / "ora.bin")
    assert (tmp_path / "ora.bin").read_bytes() == (tmp_path / "ref.bin").read_bytes()
    rng = np.random.default_rng(5)
    mu = np.where(rng.integers(0, 2, 3) == 1, 1 << 29, -(1 << 29)).astype(np.int64)
    lwe = ref.encrypt(mu)
    v = lutmod.sign_lut(p.N, p.torus_bits)
    np.testing.assert_array_equal(ora.pbs_wwl24(lwe, v), ref.pbs_wwl24(lwe, v))

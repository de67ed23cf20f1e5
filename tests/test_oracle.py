"""CPU tests of the oracle: the plain-C restatement against the reference's own code, the
reference's known-answer vectors, and the committed golden fixtures.

Tests marked ``needs_reference`` compile and call the reference's sources (oracle/_ref)
and are skipped where the reference tree is absent; the golden-fixture tests run anywhere.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as o
from oracle.oracle import Restatement
from yatfhe_gb300 import lut as lutmod
from yatfhe_gb300.params import PbsParams, T32_N1024, T56_N2048, small

GOLDEN = Path(__file__).resolve().parent / "golden"
needs_reference = pytest.mark.skipif(not o.reference_available(), reason="reference tree not present")


def _ref(p):
    return o.Reference(p)


# ---------------------------------------------------------------- known-answer vectors

def test_rotation_known_answers():
    """POLY.ROT (google_tests/polynomial_rotation_test.cpp:27-65): X^i (1,2,3,4) for i in [-8, 8]
    and (X^i - 1)(1,2,3,4), N = 4."""
    p = PbsParams(n=1, N=4, k=1, radix_bits=4, l=1, l_approx=1, ks_radix_bits=2, ks_level=1, lwe_noise_b=1,
                  rlwe_noise_b=1, torus_base=4, torus_bits=32)
    ora = Restatement(p)
    zo, m1, m2, m3 = [1, 2, 3, 4], [2, 3, 4, -1], [3, 4, -1, -2], [4, -1, -2, -3]
    m4, m5, m6, m7 = [-1, -2, -3, -4], [-2, -3, -4, 1], [-3, -4, 1, 2], [-4, 1, 2, 3]
    table = {0: zo, 8: zo, 16: zo, 1: m7, 9: m7, 2: m6, 10: m6, 3: m5, 11: m5, 4: m4, 12: m4, 5: m3, 13: m3,
             6: m2, 14: m2, 7: m1, 15: m1}
    a = np.array(zo, np.int64)
    for i in range(-8, 9):
        want = np.array(table[i + 8], np.int64)
        np.testing.assert_array_equal(ora.rotate(a, i, False), want, err_msg=f"X^{i}")
        np.testing.assert_array_equal(ora.rotate(a, i, True), want - a, err_msg=f"X^{i} - 1")


# ---------------------------------------------------------------- golden fixtures

def _golden(name):
    return np.load(GOLDEN / f"{name}.npz")


def _params_of(g):
    v = [int(x) for x in g["params"]]
    return PbsParams(*v)


@pytest.mark.parametrize("name", ["t32_n1024_small40_seed7", "t32_n1024_seed5eed0001", "t56_n2048_seed5eed0003"])
def test_restatement_reproduces_reference_golden(name):
    """The restatement regenerates the reference's keys from the seed (same SHA-256) and
    its bootstrap outputs, decryptions and intermediate accumulators bit for bit."""
    import hashlib

    g = _golden(name)
    p = _params_of(g)
    ora = Restatement(p)
    ora.keygen(int(g["seed"][0]))
    s, z = ora.keys()
    h = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()  # noqa: E731
    assert h(s) == str(g["sha_lwe_s"]) and h(z) == str(g["sha_rlwe_s"])
    assert h(ora.bsk_ntt()) == str(g["sha_bsk"])
    assert h(ora.ksk()) == str(g["sha_ksk"])
    np.testing.assert_array_equal(ora.encrypt(g["mu"]), g["lwe_in"])
    out = ora.pbs(g["lwe_in"], g["lut"], threads=8)
    np.testing.assert_array_equal(out, g["lwe_out"])
    np.testing.assert_array_equal(ora.decrypt(out, int(g["base"][0])), g["decrypted"])
    acc, final = ora.blind_rotate_trace(g["lwe_in"][0], g["lut"], list(g["checkpoints"]))
    np.testing.assert_array_equal(acc, g["acc"])
    np.testing.assert_array_equal(final, g["acc_final"])


# ---------------------------------------------------------------- restatement vs reference

@needs_reference
@pytest.mark.parametrize("base", [T32_N1024, T56_N2048])
def test_keygen_and_encryption_match_reference(base):
    p = small(base, 9)
    ref, ora = _ref(p), Restatement(p)
    for seed in (0, 1, 0xDEADBEEFCAFE):
        ref.keygen(seed)
        ora.keygen(seed)
        for a, b in zip(ref.keys(), ora.keys()):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(ref.bsk_ntt(), ora.bsk_ntt())
        np.testing.assert_array_equal(ref.ksk(), ora.ksk())
        mu = np.array([0, 1, -1, 1 << 29, -(1 << 31), (1 << 31) - 1], np.int64)
        np.testing.assert_array_equal(ref.encrypt(mu), ora.encrypt(mu))


@needs_reference
@pytest.mark.parametrize("base", [T32_N1024, T56_N2048])
def test_building_blocks_match_reference(base):
    p = small(base, 11)
    ref, ora = _ref(p), Restatement(p)
    ref.keygen(3)
    ora.keygen(3)
    rng = np.random.default_rng(0)
    T = p.torus_bits
    lo, hi = -(1 << (T - 1)), (1 << (T - 1))
    poly = rng.integers(lo, hi, p.N, dtype=np.int64)
    poly[:4] = [lo, hi - 1, 0, -1]
    # negacyclic rotation, both forms, every class of rotator
    for a in (0, 1, p.N - 1, p.N, p.N + 3, 2 * p.N - 1, -1, -p.N, -2 * p.N + 1):
        for m1 in (False, True):
            np.testing.assert_array_equal(ref.rotate(poly, a, m1), ora.rotate(poly, a, m1))
    # gadget decomposition at every level count
    for levels in range(1, p.l_approx + 1):
        np.testing.assert_array_equal(ref.decompose(poly, levels), ora.decompose(poly, levels))
    for v in list(poly[:50]) + [0, 1, -1, (1 << 31) - 1, -(1 << 31), 1 << 30]:
        v32 = int(np.int64(v).astype(np.int32))
        np.testing.assert_array_equal(ref.decompose_ks(v32), ora.decompose_ks(v32))
    # NTT / INTT in the key files' convention
    np.testing.assert_array_equal(ref.ntt_forward(poly), ora.ntt_forward(poly))
    words = ref.ntt_forward(poly)
    np.testing.assert_array_equal(ref.ntt_inverse(words), ora.ntt_inverse(words))
    np.testing.assert_array_equal(ref.ntt_inverse(words), poly)
    # modulus switch, extract, key switch, external product
    mu = rng.integers(-(1 << 31), 1 << 31, 7, dtype=np.int64)
    lwe = ref.encrypt(mu)
    lwe[0, :] = np.int32(-(1 << 31))
    for c in lwe:
        np.testing.assert_array_equal(ref.modswitch(c), ora.modswitch(c))
    acc = rng.integers(lo, hi, 2 * p.N, dtype=np.int64)
    np.testing.assert_array_equal(ref.extract(acc), ora.extract(acc))
    big = ref.extract(acc)
    np.testing.assert_array_equal(ref.keyswitch(big), ora.keyswitch(big))
    for i in (0, p.n - 1):
        np.testing.assert_array_equal(ref.external_product(acc, i), ora.external_product(acc, i))


@needs_reference
def test_test_polynomials_match_reference():
    for base in (T32_N1024, T56_N2048):
        p = small(base, 3)
        ref, ora = _ref(p), Restatement(p)
        for kind in (0, 1):
            for modP in (2, 4, 8, 16):
                np.testing.assert_array_equal(ref.test_polynomial(kind, modP), ora.test_polynomial(kind, modP))
        # the LUT builder reproduces generateTestPolynomialFR given its slot values
        for modP in (4, 8, 16):
            T = p.torus_bits
            vals = np.array([((s + modP // 2) % modP - modP // 2) * ((1 << T) // modP) for s in range(modP)])
            np.testing.assert_array_equal(lutmod.box_lut(p.N, T, vals), ref.test_polynomial(1, modP))


@needs_reference
def test_bsk_file_format_interchange(tmp_path):
    """Key files written by the reference load in the restatement and vice versa, and have the
    size the format implies."""
    p = small(T32_N1024, 5)
    ref, ora = _ref(p), Restatement(p)
    ref.keygen(9)
    f1 = tmp_path / "ref.bin"
    ref.save_bsk_file(f1)
    assert f1.stat().st_size == p.bsk_file_bytes()
    ora.load_bsk_file(f1)
    np.testing.assert_array_equal(ora.bsk_ntt(), ref.bsk_ntt())
    f2 = tmp_path / "ora.bin"
    ora.save_bsk_file(f2)
    assert f1.read_bytes() == f2.read_bytes()


def test_bsk_file_size_formula_matches_reference_statement():
    """180 x 262,313 + 9 = 178,372,849 B: the GINX key size the reference quotes for its default
    TORUS32 set n=680, N=2048, l=4 (benchmark_run/satcurve_model.py:16)."""
    p = PbsParams(n=680, N=2048, k=1, radix_bits=4, l=8, l_approx=4, ks_radix_bits=2, ks_level=16, lwe_noise_b=18,
                  rlwe_noise_b=3, torus_base=4, torus_bits=32)
    assert p.bsk_file_bytes() == 178_372_849


def test_bsk_file_rejects_truncation(tmp_path):
    p = small(T32_N1024, 3)
    ora = Restatement(p)
    ora.keygen(1)
    f = tmp_path / "k.bin"
    ora.save_bsk_file(f)
    data = f.read_bytes()
    (tmp_path / "short.bin").write_bytes(data[:-100])
    with pytest.raises(RuntimeError):
        Restatement(p).load_bsk_file(tmp_path / "short.bin")


@needs_reference
@pytest.mark.parametrize("base", [T32_N1024, T56_N2048])
def test_pbs_and_trace_match_reference(base):
    p = small(base, 14)
    ref, ora = _ref(p), Restatement(p)
    ref.keygen(21)
    ora.keygen(21)
    mu = np.array([1 << 29, -(1 << 29), 0, 1 << 27], np.int64)
    lwe = ref.encrypt(mu)
    lut = ref.test_polynomial(1, 8)
    np.testing.assert_array_equal(ref.pbs(lwe, lut, threads=0), ora.pbs(lwe, lut, threads=2))
    cps = [0, 3, p.n - 1]
    a1, f1 = ref.blind_rotate_trace(lwe[1], lut, cps)
    a2, f2 = ora.blind_rotate_trace(lwe[1], lut, cps)
    np.testing.assert_array_equal(a1, a2)
    np.testing.assert_array_equal(f1, f2)


def test_decomposition_properties():
    """GADGET_DECOMP.ZERO_MEAN (google_tests/decomposition_test.cpp:48-129): |digit| <= B/2,
    decompose(-x) = -decompose(x) away from the tie boundary, and the digits recompose x to
    within the dropped precision."""
    for base in (T32_N1024, T56_N2048):
        p = small(base, 2)
        ora = Restatement(p)
        T, b, L = p.torus_bits, p.radix_bits, p.l_approx
        rng = np.random.default_rng(5)
        x = rng.integers(-(1 << (T - 1)) + 1, 1 << (T - 1), p.N, dtype=np.int64)
        d = ora.decompose(x, L)
        assert np.abs(d).max() <= (1 << (b - 1))
        g = np.array([1 << (T - (lvl + 1) * b) for lvl in range(L)], dtype=object)
        rec = (d.astype(object) * g[:, None]).sum(axis=0)
        err = np.array([int(((int(r) - int(v)) + (1 << (T - 1))) % (1 << T) - (1 << (T - 1))) for r, v in zip(rec, x)])
        assert np.abs(err).max() <= (1 << (T - L * b - 1))
        dn = ora.decompose(-x, L)
        same = np.all(dn == -d, axis=0)
        assert same.mean() > 0.99


def test_keygen_samples_reproduce_keygen():
    """keygen_samples draws the same stream as keygen and reports its samples consistently:
    the KSK masks and the secrets are the ones inside the keys."""
    p = small(T32_N1024, 4)
    a, b = Restatement(p), Restatement(p)
    a.keygen(17)
    d = b.keygen_samples(17)
    np.testing.assert_array_equal(a.bsk_ntt(), b.bsk_ntt())
    np.testing.assert_array_equal(a.ksk(), b.ksk())
    s, z = a.keys()
    np.testing.assert_array_equal(d["lwe_s"], s)
    np.testing.assert_array_equal(d["rlwe_s"], z.reshape(-1))
    ksk = a.ksk().reshape(p.k * p.N, p.ks_level, p.n + 1)
    np.testing.assert_array_equal(d["ksk_mask"], ksk[:, :, :p.n])
    assert np.abs(d["bsk_noise"]).max() < 1 << (p.rlwe_noise_b + 1)
    assert (d["bsk_mask"] < p.q_ntt).all()

"""The approximate-CRT blind rotation (blindRotateApproxCRTNtt, yatfhe/src/blind_rotate.cpp:
577-589) in the plain-C restatement, pinned against the reference's own code: its keys
(genBootstrappingKeyApproxCrt), encryptions and rotations, in the sequence of the reference's
BLIND_ROT_APPROX_CRT_NTT test (google_tests/blindrot_test.cpp:574-640); and against the
committed fixture, which needs no reference."""
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import CrtReference, crt_blind_rotate, reference_available

GOLDEN = Path(__file__).resolve().parent / "golden"
needs_ref = pytest.mark.skipif(not reference_available(), reason="reference tree not present")


def negacyclic_shift(plain, shift, base):
    N = len(plain)
    out = np.zeros(N, np.int64)
    for j in range(N):
        src, sign = j - shift, 1
        while src < 0:
            src, sign = src + N, -sign
        out[j] = sign * int(plain[src])
    return ((out + base // 2) % base) - base // 2


def test_fixture_matches_restatement():
    g = np.load(GOLDEN / "crt_n3_n2048_seed5eed0011.npz")
    out, mcrt = crt_blind_rotate(g["bsk8"], g["acc_in"], g["rot"])
    np.testing.assert_array_equal(out, g["acc_out"])
    np.testing.assert_array_equal(mcrt, g["mcrt"])
    np.testing.assert_array_equal(g["dec"], negacyclic_shift(g["plain"], int(g["shift"][0]), 4))


@needs_ref
@pytest.mark.parametrize("n,N,seed", [(5, 2048, 3), (7, 1024, 4)])
def test_restatement_matches_reference(n, N, seed):
    r = CrtReference(n, N)
    r.keygen(seed)
    bsk = r.bsk8()
    assert bsk.min() >= -125 and bsk.max() <= 125
    rng = np.random.default_rng(seed)
    plain = rng.integers(-r.base // 2, r.base // 2, N).astype(np.int32)
    ct = r.encrypt(plain)
    # negative amounts, a multiple of 2N (no rotation, not skipped by the reference) and 0
    rot = rng.integers(-3 * N, 3 * N, n).astype(np.int32)
    rot[1], rot[3] = 0, 4 * N
    want, want_mcrt = r.blind_rotate(ct, rot)
    got, got_mcrt = crt_blind_rotate(bsk, ct, rot)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(got_mcrt, want_mcrt)
    shift = int((rot.astype(np.int64) * r.lwe_key()).sum()) % (2 * N)
    np.testing.assert_array_equal(r.decrypt(got), negacyclic_shift(plain, shift, r.base))


@needs_ref
def test_ntt_and_coefficient_rotations_agree_on_the_reference():
    """blindRotateApproxCRT (schoolbook products mod q_d) and blindRotateApproxCRTNtt (products
    mod 2^24 - 2^14 + 1, then mod q_d) agree whenever no product sum reaches half that prime,
    which is every case here; the restatement follows the NTT form."""
    r = CrtReference(3, 1024)
    r.keygen(9)
    rng = np.random.default_rng(9)
    ct = r.encrypt(rng.integers(-2, 2, 1024).astype(np.int32))
    rot = rng.integers(1, 2048, 3).astype(np.int32)
    a, _ = r.blind_rotate(ct, rot, ntt=True)
    b, _ = r.blind_rotate(ct, rot, ntt=False)
    np.testing.assert_array_equal(a, b)

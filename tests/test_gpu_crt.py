"""The approximate-CRT blind rotation on the GPU (yg_crt_blind_rotate): equal to the
reference's own output in the committed fixture, and to the restatement (pinned to the
reference by tests/test_crt_oracle.py) on random residue keys, rotations and samples at both
ring sizes and at the reference's default size (n = 680, N = 2048)."""
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import CRT_Q, crt_blind_rotate

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def random_case(n, N, count, seed):
    rng = np.random.default_rng(seed)
    # residues centred mod each prime, as decompTrgswMcrt leaves them
    bsk8 = np.empty((n, 4, 2, 2, 2, N), np.int8)
    for d, q in enumerate((251, 241, 239, 233)):
        bsk8[:, d] = rng.integers(-(q // 2), q // 2 + 1, size=bsk8[:, d].shape)
    acc = rng.integers(-(CRT_Q // 2), CRT_Q // 2 + 1, size=(count, 2, N)).astype(np.int32)
    rot = rng.integers(-4 * N, 4 * N, size=(count, n)).astype(np.int32)
    rot[:, ::5] = 0
    return bsk8, acc, rot


def test_matches_reference_fixture(built_lib):
    from yatfhe_gb300 import api

    g = np.load(GOLDEN / "crt_n3_n2048_seed5eed0011.npz")
    key = api.CrtKey(g["bsk8"])
    out = key.blind_rotate(torch.from_numpy(g["acc_in"][None]).cuda(), torch.from_numpy(g["rot"][None]).cuda())
    np.testing.assert_array_equal(out.cpu().numpy()[0], g["acc_out"])


@pytest.mark.parametrize("n,N,count", [(24, 2048, 5), (40, 1024, 7)])
def test_matches_restatement(n, N, count, built_lib):
    from yatfhe_gb300 import api

    bsk8, acc, rot = random_case(n, N, count, n + N)
    key = api.CrtKey(bsk8)
    assert key.device_bytes == n * 16 * 2 * N * 4
    out = key.blind_rotate(torch.from_numpy(acc).cuda(), torch.from_numpy(rot).cuda()).cpu().numpy()
    for c in range(count):
        want, _ = crt_blind_rotate(bsk8, acc[c], rot[c])
        np.testing.assert_array_equal(out[c], want)


def test_default_size_and_edges(built_lib):
    from yatfhe_gb300 import api

    n, N = 680, 2048
    bsk8, acc, rot = random_case(n, N, 3, 7)
    rot[1] = 0  # every step skipped: the conversions alone
    key = api.CrtKey(bsk8)
    d_acc, d_rot = torch.from_numpy(acc).cuda(), torch.from_numpy(rot).cuda()
    out = key.blind_rotate(d_acc, d_rot).cpu().numpy()
    for c in (0, 1):
        want, _ = crt_blind_rotate(bsk8, acc[c], rot[c])
        np.testing.assert_array_equal(out[c], want)
    np.testing.assert_array_equal(out[1], acc[1])  # decomposition and recomposition invert each other
    # an empty batch, and a residue outside every prime's range
    key.blind_rotate(d_acc[:0], d_rot[:0])
    bad = bsk8[:2].copy()
    bad[0, 0, 0, 0, 0, 5] = -128
    with pytest.raises(Exception, match="outside"):
        api.CrtKey(bad)


def test_persistent_grid_covers_every_ciphertext(built_lib):
    """More ciphertexts than resident CTAs (two per SM): the grid loops, and ciphertexts of
    every round equal the restatement."""
    from yatfhe_gb300 import api

    n, N = 6, 1024
    count = 2 * torch.cuda.get_device_properties(0).multi_processor_count * 2 + 37
    bsk8, acc, rot = random_case(n, N, count, 99)
    key = api.CrtKey(bsk8)
    out = key.blind_rotate(torch.from_numpy(acc).cuda(), torch.from_numpy(rot).cuda()).cpu().numpy()
    for c in sorted({0, 1, count // 2, count // 2 + 1, count - 2, count - 1}):
        want, _ = crt_blind_rotate(bsk8, acc[c], rot[c])
        np.testing.assert_array_equal(out[c], want)

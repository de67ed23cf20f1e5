"""yg_pbs_noalloc, the bootstrap entry point that allocates nothing.

It exists for callers that cannot let a library allocate device memory: programs whose
GPU memory is owned by their own allocator or a fixed budget, and services that reserve
all memory at start-up and treat later allocations as faults.  It keeps the intermediate
ciphertexts in a fixed array compiled into the library instead of a per-call buffer.

Checked here through the C ABI: two calls in a row (the second sees the first call's
leftovers in the shared array) return exactly what the allocating yg_pbs returns, and a
call larger than the fixed array is rejected.  This file is collected last so that a run
stopping at the first failure has already run every other test; it also passes alone.
"""
import ctypes

import numpy as np
import pytest

from oracle.oracle import Restatement
from yatfhe_gb300.params import T32_N1024, small

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_allocating_entry_point_twice(built_lib):
    from yatfhe_gb300 import _lib, api

    p = small(T32_N1024, 40)
    ora = Restatement(p)
    ora.keygen(0xA110C)
    ctx = api.Context(p, 0)
    key = api.BootstrapKey.from_ntt_words(ctx, ora.bsk_ntt()).set_ksk(ora.ksk())
    L = _lib.lib()
    max_count = int(L.yg_pbs_noalloc_max_count(ctx.handle))
    assert max_count == (4 << 20) // (p.N + 1)

    rng = np.random.default_rng(9)
    lut = torch.from_numpy(np.full(p.N, 1 << 29, np.int64)).cuda()
    stream = torch.cuda.current_stream()
    sh = ctypes.c_void_p(stream.cuda_stream)
    for count in (257, max_count):  # two calls in a row, the second at the size limit
        lwe = rng.integers(-(1 << 31), 1 << 31, size=(count, p.n + 1), dtype=np.int64).astype(np.int32)
        d_in = torch.from_numpy(lwe).cuda()
        want = torch.empty_like(d_in)
        got = torch.full_like(d_in, -1)
        _lib.check(L.yg_pbs(ctx.handle, key.handle, _vp(d_in), _vp(want), count, _vp(lut), sh))
        _lib.check(L.yg_pbs_noalloc(ctx.handle, key.handle, _vp(d_in), _vp(got), count, _vp(lut), sh))
        torch.cuda.synchronize()
        assert torch.equal(got, want), f"no-alloc bootstrap differs from yg_pbs at count={count}"

    # spot check against the oracle too
    np.testing.assert_array_equal(got[:3].cpu().numpy(), ora.pbs(lwe[:3], lut.cpu().numpy()))

    too_many = max_count + 1
    d_in = torch.zeros((too_many, p.n + 1), dtype=torch.int32, device="cuda")
    d_out = torch.empty_like(d_in)
    rc = L.yg_pbs_noalloc(ctx.handle, key.handle, _vp(d_in), _vp(d_out), too_many, _vp(lut), sh)
    assert rc == -1
    assert b"exceed the fixed scratch" in L.yg_last_error()

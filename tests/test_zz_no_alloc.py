"""yg_pbs_noalloc, the bootstrap entry point that allocates nothing.

It exists for callers that cannot let a library allocate device memory: programs whose
GPU memory is owned by their own allocator or a fixed budget, and services that reserve
all memory at start-up and treat later allocations as faults.  It keeps the intermediate
ciphertexts in a fixed array compiled into the library instead of a per-call buffer.

Checked here through the C ABI: after the set-up call (count 0), two calls in a row (the
second sees the first call's leftovers in the shared array) return exactly what the
allocating yg_pbs returns, while the device's free memory and the stream-ordered pool's
high-water mark stay where they were (the same probe sees yg_pbs's own allocation, so it
would see one); a call larger than the fixed array is rejected.  This file is collected
last so that a run stopping at the first failure has already run every other test; it
also passes alone.
"""
import ctypes
import ctypes.util
import glob
import os

import numpy as np
import pytest

from oracle.oracle import Restatement
from yatfhe_gb300.params import T32_N1024, small

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

_ATTR_USED_MEM_HIGH = 8  # cudaMemPoolAttrUsedMemHigh


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _cudart():
    """The CUDA runtime as a shared library, for the stream-ordered pool's counters (the
    pool is a driver object per device, the same whichever runtime copy asks)."""
    cands = [ctypes.util.find_library("cudart")]
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d:
            cands += sorted(glob.glob(os.path.join(d, "lib64", "libcudart.so*")))
    for c in cands:
        if not c:
            continue
        try:
            return ctypes.CDLL(c)
        except OSError:
            continue
    return None


class _Pool:
    """High-water mark of the device's default stream-ordered memory pool."""

    def __init__(self, rt, device):
        self.rt = rt
        self.pool = ctypes.c_void_p()
        assert rt.cudaDeviceGetDefaultMemPool(ctypes.byref(self.pool), device) == 0

    def reset(self):
        zero = ctypes.c_uint64(0)
        assert self.rt.cudaMemPoolSetAttribute(self.pool, _ATTR_USED_MEM_HIGH, ctypes.byref(zero)) == 0

    def high(self):
        v = ctypes.c_uint64(0)
        assert self.rt.cudaMemPoolGetAttribute(self.pool, _ATTR_USED_MEM_HIGH, ctypes.byref(v)) == 0
        return v.value


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
    rt = _cudart()
    pool = _Pool(rt, 0) if rt is not None else None

    # every buffer of the test first, so that nothing below but the library could allocate
    counts = (257, max_count)  # two calls in a row, the second at the size limit
    lwes = [rng.integers(-(1 << 31), 1 << 31, size=(c, p.n + 1), dtype=np.int64).astype(np.int32) for c in counts]
    d_ins = [torch.from_numpy(x).cuda() for x in lwes]
    wants = [torch.empty_like(d) for d in d_ins]
    gots = [torch.full_like(d, -1) for d in d_ins]
    for count, d_in, want in zip(counts, d_ins, wants):
        if pool is not None:
            pool.reset()
        _lib.check(L.yg_pbs(ctx.handle, key.handle, _vp(d_in), _vp(want), count, _vp(lut), sh))
        torch.cuda.synchronize()
        if pool is not None:  # the probe sees the allocating entry point's buffer
            assert pool.high() >= count * (p.N + 1) * 4

    # set-up: the array's address looked up (its memory committed) and the kernels loaded
    _lib.check(L.yg_pbs_noalloc(ctx.handle, key.handle, None, None, 0, None, sh))
    torch.cuda.synchronize()

    free_before = torch.cuda.mem_get_info(0)[0]
    if pool is not None:
        pool.reset()
    for count, d_in, got in zip(counts, d_ins, gots):
        _lib.check(L.yg_pbs_noalloc(ctx.handle, key.handle, _vp(d_in), _vp(got), count, _vp(lut), sh))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free_before, "device free memory changed across yg_pbs_noalloc calls"
    if pool is not None:
        assert pool.high() == 0, "yg_pbs_noalloc took memory from the stream-ordered pool"
    for count, got, want in zip(counts, gots, wants):
        assert torch.equal(got, want), f"no-alloc bootstrap differs from yg_pbs at count={count}"

    # spot check against the oracle too
    np.testing.assert_array_equal(gots[-1][:3].cpu().numpy(), ora.pbs(lwes[-1][:3], lut.cpu().numpy()))

    too_many = max_count + 1
    d_in = torch.zeros((too_many, p.n + 1), dtype=torch.int32, device="cuda")
    d_out = torch.empty_like(d_in)
    rc = L.yg_pbs_noalloc(ctx.handle, key.handle, _vp(d_in), _vp(d_out), too_many, _vp(lut), sh)
    assert rc == -1
    assert b"exceed the fixed scratch" in L.yg_last_error()

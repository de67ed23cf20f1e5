"""Multi-rank host logic on CPU: world_size-2 gloo ranks shard independent bootstraps and
agree on the max-over-ranks time, with no collective on the data path."""
import os
import socket

import numpy as np
import pytest

from yatfhe_gb300.shard import shard_range, shard_tenants


def test_shard_range_partitions_exactly():
    for count in (0, 1, 7, 65536, 65537):
        for world in (1, 2, 3, 8):
            spans = [shard_range(count, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == count
            for (a, b), (c, d) in zip(spans, spans[1:]):
                assert b == c
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def test_shard_tenants_disjoint_cover():
    ids = list(range(1, 33))
    parts = [shard_tenants(ids, r, 4) for r in range(4)]
    assert sorted(sum(parts, [])) == ids


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist

    from oracle.oracle import Restatement
    from yatfhe_gb300.params import T32_N1024, small
    from yatfhe_gb300.shard import max_over_ranks, shard_range

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        p = small(T32_N1024, 6)
        ora = Restatement(p)
        ora.keygen(77)  # same key on every rank (tenant replicated for this test)
        mu = np.array([(1 if i % 3 else -1) << 29 for i in range(10)], np.int64)
        lwe = ora.encrypt(mu)
        b, e = shard_range(len(lwe), rank, world)
        out = ora.pbs(lwe[b:e], np.full(p.N, 1 << 29, np.int64))
        t = max_over_ranks(float(rank + 1))
        q.put((rank, b, e, out, t))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_agree_on_max_time():
    import torch.multiprocessing as mp

    from oracle.oracle import Restatement
    from yatfhe_gb300.params import T32_N1024, small

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = [q.get(timeout=120) for _ in procs]
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    res.sort()
    assert [r[4] for r in res] == [2.0, 2.0]
    # the shards reassemble the single-process result
    p = small(T32_N1024, 6)
    ora = Restatement(p)
    ora.keygen(77)
    mu = np.array([(1 if i % 3 else -1) << 29 for i in range(10)], np.int64)
    lwe = ora.encrypt(mu)
    whole = ora.pbs(lwe, np.full(p.N, 1 << 29, np.int64))
    np.testing.assert_array_equal(np.concatenate([r[3] for r in res]), whole)

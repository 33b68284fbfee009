"""Multi-GPU partition by code range (ugsdr_gb300/sharding.py), host side:
world_size 2 over gloo on the CPU, each rank searching its share of the codes
with the oracle's acquisition (the device search is the same call on each
rank's own GPU); the gathered records must equal one process searching all
codes."""
import os
import socket

import numpy as np
import pytest

from conftest import GOLDEN, unpack_codes
from ugsdr_gb300 import sharding

FS, N, K = 4e6, 4000, 2


def test_code_range_partition():
    for n in (0, 1, 5, 32, 37, 63):
        for w in (1, 2, 3, 8):
            ranges = [sharding.code_range(n, r, w) for r in range(w)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(b == c for (_, b), (c, _) in zip(ranges, ranges[1:]))
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)
    assert sharding.shard(list(range(5)), 1, 2) == [3, 4]
    with pytest.raises(ValueError):
        sharding.code_range(4, 2, 2)
    with pytest.raises(ValueError):
        sharding.code_range(4, 0, 0)


def case():
    from ugsdr_gb300 import signals
    ca = unpack_codes(np.load(GOLDEN / "codes.npz"), "gps_l1ca")
    codes = {p: ca[p] for p in range(7)}
    raw, _ = signals.gps_l1_config(seed=3, codes=codes, fs=FS, ms=N * K // 4000, visible=3, sample_type="ci8")
    x = raw.astype(np.float32)
    return (x[:, 0] + 1j * x[:, 1]).astype(np.complex64), codes


def search_codes(x, codes, prns):
    import pyoracle
    out = []
    for p in prns:
        rec = pyoracle.acquire(x, N, K, pyoracle.upsample(codes[p], N), FS, 2000, 500)
        out.append((p, int(rec["index"]), int(rec["doppler_bin"]), float(rec["level"]), float(rec["snr"])))
    return out


def worker(rank, world, port, queue):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        x, codes = case()
        prns = sorted(codes)
        res = sharding.search(prns, rank, world, lambda share: search_codes(x, codes, share))
        queue.put((rank, res))
    finally:
        dist.destroy_process_group()


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_search_equals_one():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(queue.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    x, codes = case()
    whole = search_codes(x, codes, sorted(codes))
    assert got[0] == whole and got[1] == whole

"""Pass sharding over ranks: block assignment, and the gloo reduction of
per-rank image sums equals the single-process average (world size 2 and 3,
CPU; a stand-in renderer whose pass images depend on the pass index)."""
import os
import socket

import numpy as np
import pytest

from ppmpa_gb300.shard import render_sharded, shard_passes, torch_reduce_sum


def test_blocks_cover_every_pass_once():
    for total in (0, 1, 5, 64, 65):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                first, count = shard_passes(total, r, world)
                seen += list(range(first, first + count))
            assert seen == list(range(total))
    with pytest.raises(ValueError):
        shard_passes(4, 2, 2)


def _pass_image(k):
    rng = np.random.default_rng(1000 + k)
    return rng.random((4, 5, 3)) * (k + 1) ** -0.5


def _stand_in(first, count):
    return sum(_pass_image(k) for k in range(first, first + count))


def _worker(rank, world, port, total, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        img = render_sharded(_stand_in, total, rank, world, torch_reduce_sum())
        q.put((rank, img))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world,total", [(2, 7), (3, 10)])
def test_gloo_sharded_average_equals_single_process(world, total):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, total, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want = _stand_in(0, total) / total
    assert all(out[r] is None for r in range(1, world))
    assert np.allclose(out[0], want, rtol=1e-13, atol=0)

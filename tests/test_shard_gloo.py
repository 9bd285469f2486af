"""Pass sharding over ranks (host side, two gloo ranks on CPU): the passes of
one image are dealt round robin, every pass to exactly one rank, and the
per-rank accumulation buffers merge into the image of all passes with one
sum over the ranks."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import pppm_gb300 as P


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, total, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = P.shard_passes(total, rank, world)
        # a stand-in accumulation: each pass t adds t to every pixel
        acc = np.zeros((4, 5, 3), np.float32)
        for t in mine:
            acc += t
        img = P.merge_shards(acc, total)
        got = [None] * world
        dist.all_gather_object(got, mine)
        if rank == 0:
            out.put((got, img))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("total", [1, 6, 7])
def test_two_ranks_merge_to_the_full_image(total):
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, total, q)) for r in range(world)]
    for p in procs:
        p.start()
    got, img = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    flat = sorted(t for lst in got for t in lst)
    assert flat == list(range(1, total + 1))
    np.testing.assert_allclose(img, np.full((4, 5, 3), sum(range(1, total + 1)) / total), rtol=1e-6)


def test_shard_passes_bad_rank():
    with pytest.raises(ValueError):
        P.shard_passes(4, 2, 2)

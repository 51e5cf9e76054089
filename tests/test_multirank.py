"""The multi-GPU host logic on CPU: two gloo ranks on 127.0.0.1 split a
batch of worlds, and the whole-job rate takes the sum of the ranks' work over
the slowest rank's time. No GPU and no data-path collective are involved."""
import os
import socket

import numpy as np
import pytest

from nphysics_gb300 import multirank, scenes


def test_shard_covers_every_item_once():
    for n in (0, 1, 7, 4096, 4097):
        for ws in (1, 2, 3, 8):
            got = [i for r in range(ws) for i in multirank.shard(n, r, ws)]
            assert got == list(range(n))
            lens = [len(multirank.shard(n, r, ws)) for r in range(ws)]
            assert max(lens) - min(lens) <= 1
    with pytest.raises(ValueError):
        multirank.shard(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world_size, port, n_worlds, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world_size))
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    try:
        r, ws, _ = multirank.rank_env()
        mine = multirank.shard(n_worlds, r, ws)
        sc = scenes.batched_worlds(n_worlds=n_worlds, lo=8, hi=40, worlds=mine)
        dyn = int((sc.bodies["status"] == 2).sum())
        seconds = 1.0 + r            # rank 1 is the slow one
        rate = multirank.whole_job_rate(dyn, seconds)
        total = multirank.reduce_sum(dyn)
        np.save(os.path.join(out_dir, f"rank{r}.npy"),
                np.array([mine.start, mine.stop, dyn, total, rate, sc.bodies["world"].max()]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_split_a_batch(tmp_path):
    import torch.multiprocessing as mp
    n_worlds = 24
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, n_worlds, str(tmp_path)), nprocs=2, start_method="spawn")
    r0, r1 = (np.load(tmp_path / f"rank{r}.npy") for r in range(2))
    assert (r0[0], r0[1], r1[0], r1[1]) == (0, 12, 12, 24)
    whole = scenes.batched_worlds(n_worlds=n_worlds, lo=8, hi=40)
    n_dyn = int((whole.bodies["status"] == 2).sum())
    assert r0[2] + r1[2] == n_dyn
    assert r0[3] == r1[3] == n_dyn
    assert r0[4] == pytest.approx(n_dyn / 2.0)      # slowest rank: 2 s
    assert r0[5] == r1[5] == 11                      # worlds renumbered from 0 on each rank

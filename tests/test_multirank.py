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


def _bench_rank_main(rank, world_size, port, out_dir):
    # bench.py's whole-job reduction, as each rank of a multi-GPU run calls it
    # (gloo on the CPU instead of NCCL): rank r processed 100 + 50 r bodies in
    # 4 + 3 r ms of device time and 1 + r s end to end.
    import sys

    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world_size))
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    try:
        value, e2e, ms = bench.whole_job(100 + 50 * rank, 4.0 + 3.0 * rank, 1.0 + rank, device=None)
        np.save(os.path.join(out_dir, f"bench{rank}.npy"), np.array([value, e2e, ms]))
    finally:
        dist.destroy_process_group()


def test_bench_whole_job_reduction_under_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_bench_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    for r in range(2):
        value, e2e, ms = np.load(tmp_path / f"bench{r}.npy")
        assert ms == 7.0                                  # the slowest rank's device time
        assert value == pytest.approx(250 / 7e-3)         # all ranks' bodies over it
        assert e2e == pytest.approx(250 / 2.0)


def test_bench_reference_arm_under_torchrun():
    # The driver launches the reference arm with torchrun at N > 1: rank 0
    # alone times the oracle and prints one line, the other rank exits 0.
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    port = _free_port()
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "0", "--settle", "1", "--side", "4"],
                       cwd=root, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2


def test_sharded_batch_steps_like_the_whole_batch():
    # The colouring hashes world-local collider slots, so a world steps to the
    # same bits whether it sits in the whole batch or in a rank's shard (the
    # oracle in the GPU's colour order; the GPU twin is in test_gpu_batched).
    from oracle.oracle_py import ORDER_COLOUR, OracleWorld

    def run(sc):
        o = OracleWorld(sc.params(), sc.gravity, precision=32, order=ORDER_COLOUR)
        o.load_scene(sc)
        o.step(60)
        return o.bodies()
    n = 8
    whole = run(scenes.batched_worlds(n_worlds=n, seed=3, lo=8, hi=120))
    shards = [run(scenes.batched_worlds(n_worlds=n, seed=3, lo=8, hi=120, worlds=multirank.shard(n, r, 2)))
              for r in range(2)]
    for k in ("position", "velocity", "active"):
        np.testing.assert_array_equal(whole[k], np.concatenate([s[k] for s in shards]))

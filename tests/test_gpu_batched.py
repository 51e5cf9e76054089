"""Batched worlds: the block-per-world schedule against the one-grid schedule
and the oracle.

Many independent worlds of uneven size, each on its own ground. Both GPU
schedules visit every body's manifolds in colour order, so they must agree
bit for bit; the oracle's colour order is the same sequence on the CPU.
"""
import numpy as np
import pytest

from nphysics_gb300 import abi, scenes
from oracle.oracle_py import ORDER_COLOUR, OracleWorld

pytestmark = pytest.mark.gpu


def run(scene, schedule, steps):
    from nphysics_gb300.world import GpuWorld
    p = scene.params()
    p.solver_schedule = schedule
    g = GpuWorld.for_scene(scene, p)
    g.step(steps)
    return g


def small_batch(n_worlds=10, seed=7):
    return scenes.batched_worlds(n_worlds=n_worlds, seed=seed, lo=8, hi=120)


@pytest.mark.parametrize("hi", [120, 700])
def test_worlds_schedule_equals_grid_schedule(gpu_lib, hi):
    # hi 120: every world is solved by one warp; hi 700: the worlds wider than
    # 256 body slots take a whole block, the rest a warp.
    sc = scenes.batched_worlds(n_worlds=10, seed=7, lo=8, hi=hi)
    a = run(sc, abi.SCHEDULE_GRID, 40)
    b = run(sc, abi.SCHEDULE_WORLDS, 40)
    ba, bb = a.bodies(), b.bodies()
    np.testing.assert_array_equal(ba["position"], bb["position"])
    np.testing.assert_array_equal(ba["velocity"], bb["velocity"])
    np.testing.assert_array_equal(a.pairs(), b.pairs())
    ca, cb = a.counters(), b.counters()
    assert ca["num_constraints"] == cb["num_constraints"] > 0
    assert ca["velocity_iterations"] == cb["velocity_iterations"]
    # FP64 sums in a different order.
    assert abs(ca["residual"] - cb["residual"]) <= 1e-12 + 1e-9 * abs(ca["residual"])


def test_cluster_worlds_mixed_with_block_worlds(gpu_lib):
    # Worlds wider than 4096 body slots are solved by a thread-block cluster
    # (Δv in distributed shared memory), the others by a block or a warp, in
    # the same step; the bits are the one grid's.
    sc = scenes.batched_worlds(n_worlds=5, seed=3, lo=200, hi=9000)
    widths = np.bincount(sc.bodies["world"])
    assert (widths > 4097).any() and (widths <= 4097).any()
    a = run(sc, abi.SCHEDULE_GRID, 30)
    b = run(sc, abi.SCHEDULE_WORLDS, 30)
    ba, bb = a.bodies(), b.bodies()
    np.testing.assert_array_equal(ba["position"], bb["position"])
    np.testing.assert_array_equal(ba["velocity"], bb["velocity"])


def test_worlds_schedule_matches_oracle(gpu_lib):
    sc = small_batch(n_worlds=6, seed=3)
    g = run(sc, abi.SCHEDULE_WORLDS, 25)
    o = OracleWorld(sc.params(), sc.gravity, precision=32, order=ORDER_COLOUR)
    o.load_scene(sc)
    o.step(25)
    gb, ob = g.bodies(), o.bodies()
    err = np.abs(gb["position"].astype(np.float64) - ob["position"])
    assert err.max() <= 1e-5 + 1e-5 * np.abs(ob["position"]).max(), err.max()
    np.testing.assert_array_equal(g.pairs(), o.pairs())


def test_interleaved_worlds_fall_back_to_grid(gpu_lib):
    # World indices that are not contiguous in slot order cannot run one block
    # per world; the step still runs (on the grid schedule) and matches it.
    sc = small_batch(n_worlds=4, seed=9)
    b = sc.bodies.copy()
    w = b["world"].copy()
    b["world"] = w[::-1].copy()          # reverse the world order over the slots
    inter = scenes.Scene("interleaved", b, sc.colliders)
    a = run(inter, abi.SCHEDULE_GRID, 15)
    c = run(inter, abi.SCHEDULE_WORLDS, 15)
    np.testing.assert_array_equal(a.bodies()["position"], c.bodies()["position"])


def test_world_ranges_follow_removals(gpu_lib):
    # Removing every body of one world leaves an empty world in the middle of
    # the batch; the per-world schedule must keep matching the grid schedule.
    sc = small_batch(n_worlds=5, seed=21)
    worlds = sc.bodies["world"]
    gone = np.nonzero(worlds == 2)[0]
    res = []
    for sched in (abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS):
        g = run(sc, sched, 5)
        g.remove_bodies(sc.body_handles[gone])
        g.step(10)
        res.append(g.bodies()["position"])
    np.testing.assert_array_equal(res[0], res[1])


@pytest.mark.parametrize("sched", [abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS])
def test_sharded_batch_matches_the_whole_batch(gpu_lib, sched):
    # A batch sharded over two ranks, each shard stepped as its own world
    # object (here one after the other on one GPU), gives every world the same
    # bits as stepping the whole batch at once: worlds never interact and the
    # colouring hashes world-local collider slots.
    from nphysics_gb300 import multirank
    from nphysics_gb300.world import GpuWorld
    n = 64

    def run(sc):
        p = sc.params()
        p.solver_schedule = sched
        w = GpuWorld.for_scene(sc, p, pairs_per_collider=8)
        w.step(60)
        b = w.bodies()
        w.close()
        return b
    whole = run(scenes.batched_worlds(n_worlds=n, seed=9, lo=16, hi=400))
    shards = [run(scenes.batched_worlds(n_worlds=n, seed=9, lo=16, hi=400, worlds=multirank.shard(n, r, 2)))
              for r in range(2)]
    for k in ("position", "velocity", "active"):
        np.testing.assert_array_equal(whole[k], np.concatenate([s[k] for s in shards]))

"""Steps replayed from CUDA graphs give the same bits as steps launched one
kernel at a time, including across changes that force a new capture."""
import numpy as np
import pytest

from nphysics_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def run(scene, use_graph, steps, schedule=abi.SCHEDULE_AUTO, edit_at=None):
    from nphysics_gb300.world import GpuWorld
    p = scene.params()
    p.use_graph = use_graph
    p.solver_schedule = schedule
    g = GpuWorld.for_scene(scene, p)
    replays = 0
    for k in range(steps):
        if edit_at is not None and k == edit_at:
            # Push every dynamic body up by 1 m/s: new uploads, a fresh
            # start-of-step collision detection, then graphs again.
            dyn = np.nonzero(scene.bodies["status"] == abi.BODY_DYNAMIC)[0]
            f = np.zeros((len(dyn), 6), np.float32)
            f[:, 1] = 60.0
            g.apply_forces(np.ascontiguousarray(scene.body_handles[dyn]), f, wake=True)
        g.step(1)
        replays += g.counters()["graph_replay"]
    return g, replays


@pytest.mark.parametrize("which", ["pile", "worlds"])
def test_graph_steps_match_eager_steps(gpu_lib, which):
    if which == "pile":
        sc, sched = scenes.ball_pile(side=6), abi.SCHEDULE_AUTO
    else:
        sc, sched = scenes.batched_worlds(n_worlds=6, seed=4, lo=8, hi=60), abi.SCHEDULE_WORLDS
    a, ra = run(sc, 0, 60, sched, edit_at=30)
    b, rb = run(sc, 1, 60, sched, edit_at=30)
    assert ra == 0
    assert rb >= 50
    np.testing.assert_array_equal(a.bodies()["position"], b.bodies()["position"])
    np.testing.assert_array_equal(a.bodies()["velocity"], b.bodies()["velocity"])
    np.testing.assert_array_equal(a.pairs(), b.pairs())


def test_autotune_keeps_the_bits(gpu_lib):
    # The tuner advances the world by real steps under each candidate launch
    # shape; since every shape computes the same bits, the tuned world equals
    # one stepped the same number of times without tuning.
    from nphysics_gb300.world import GpuWorld
    sc = scenes.batched_worlds(n_worlds=8, seed=2, lo=8, hi=80)
    a = GpuWorld.for_scene(sc)
    sched, threads, ms = a.autotune(steps_per_candidate=3)
    assert sched in (abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS) and ms > 0
    a.step(10)
    b = GpuWorld.for_scene(sc)
    b.step(1 + 4 * (1 + 3) + 10)      # the sizing step, one grid and three world-block candidates
    np.testing.assert_array_equal(a.bodies()["position"], b.bodies()["position"])
    np.testing.assert_array_equal(a.bodies()["velocity"], b.bodies()["velocity"])

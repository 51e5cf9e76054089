"""Parity at the benchmark's own sizes.

The 32^3 ball pile (C2) is stepped on the GPU, under both solver schedules,
and by the oracle in the colour order, and they agree bit for bit, pair set
included. A batch of a few
hundred worlds of the batched-worlds scene (C4's recipe) gives the same bits
under the one-grid and the per-world schedules. The 100 000-body mixed pile
(C3: balls and cuboids dropped from heights U(1, 60) over a 100 x 100
footprint) is stepped 60 steps by the GPU and the oracle, bit for bit."""
import numpy as np
import pytest

from nphysics_gb300 import abi, scenes
from oracle.oracle_py import ORDER_COLOUR, OracleWorld

pytestmark = pytest.mark.gpu


def test_ball_pile_32k_matches_oracle(gpu_lib):
    # Both schedules: the one cooperative grid, and the per-world schedule,
    # where the pile is one world solved by a thread-block cluster.
    from nphysics_gb300.world import GpuWorld
    sc = scenes.ball_pile(side=32)
    o = OracleWorld(sc.params(), sc.gravity, precision=32, order=ORDER_COLOUR)
    o.load_scene(sc)
    o.step(100)
    ob = o.bodies()
    for sched in (abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS):
        p = sc.params()
        p.solver_schedule = sched
        g = GpuWorld.for_scene(sc, p)
        g.step(100)
        assert g.counters()["num_contacts"] > 30000      # most of the pile has landed
        np.testing.assert_array_equal(g.pairs(), o.pairs())
        gb = g.bodies()
        np.testing.assert_array_equal(gb["position"], ob["position"])
        np.testing.assert_array_equal(gb["velocity"], ob["velocity"])
        del g


def test_mixed_pile_100k_matches_oracle(gpu_lib):
    # 60 steps: the lowest bodies have landed, tumbled and piled up (about 20k
    # contacts, 8 colours, boxes on boxes and balls); the oracle takes about
    # 1.4 s a step at this size.
    from nphysics_gb300.world import GpuWorld
    sc = scenes.mixed_pile(n=100_000)
    o = OracleWorld(sc.params(), sc.gravity, precision=32, order=ORDER_COLOUR)
    o.load_scene(sc)
    o.step(60)
    ob = o.bodies()
    oc = o.counters()
    assert oc["num_contacts"] > 10000
    for sched in (abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS):
        p = sc.params()
        p.solver_schedule = sched
        g = GpuWorld.for_scene(sc, p, pairs_per_collider=12)
        g.step(60)
        gc = g.counters()
        for k in ("num_pairs", "num_manifolds", "num_contacts", "num_solver_contacts", "num_colours"):
            assert gc[k] == oc[k], k
        np.testing.assert_array_equal(g.pairs(), o.pairs())
        gb = g.bodies()
        np.testing.assert_array_equal(gb["position"], ob["position"])
        np.testing.assert_array_equal(gb["velocity"], ob["velocity"])
        del g


def test_batched_worlds_schedules_agree_at_scale(gpu_lib):
    from nphysics_gb300.world import GpuWorld
    sc = scenes.batched_worlds(n_worlds=256, seed=11)
    out = []
    for sched in (abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS):
        p = sc.params()
        p.solver_schedule = sched
        w = GpuWorld.for_scene(sc, p, pairs_per_collider=6)
        w.step(40)
        c = w.counters()
        assert c["num_constraints"] > 100000
        out.append((w.bodies()["position"], w.bodies()["velocity"], w.pairs()))
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)

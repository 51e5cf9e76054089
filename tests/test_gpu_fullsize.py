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
from oracle.oracle_py import ORDER_COLOUR, ORDER_REFERENCE, OracleWorld

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
    # The f64 oracle in the reference's order beside it: the pile is chaotic,
    # so the bounds are on statistics. Measured: kinetic energy within 1.7e-4
    # relative at every step, the maximum penetration 0.282 m against 0.279 m
    # (0.046 m apart at worst on one step), contacts within 0.8 %.
    r = OracleWorld(sc.params(), sc.gravity, precision=64, order=ORDER_REFERENCE)
    r.load_scene(sc)
    ke_o, ke_r, pen_o, pen_r, nc_o, nc_r = [], [], [], [], [], []
    for _ in range(60):
        o.step(1)
        r.step(1)
        co, cr = o.counters(), r.counters()
        ke_o.append(co["kinetic_energy"])
        ke_r.append(cr["kinetic_energy"])
        pen_o.append(co["max_penetration"])
        pen_r.append(cr["max_penetration"])
        nc_o.append(co["num_contacts"])
        nc_r.append(cr["num_contacts"])
    ke_o, ke_r = np.array(ke_o), np.array(ke_r)
    assert np.max(np.abs(ke_o - ke_r) / ke_r) <= 5e-4
    assert abs(max(pen_o) - max(pen_r)) <= 0.02
    assert np.max(np.abs(np.array(pen_o) - np.array(pen_r))) <= 0.08
    assert np.max(np.abs(np.array(nc_o) - np.array(nc_r)) / np.maximum(np.array(nc_r), 1)) <= 0.02
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

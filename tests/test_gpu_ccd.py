"""Continuous collision detection on the GPU against the oracle (through the
C ABI): MechanicalWorld::solve_ccd (src/world/mechanical_world.rs:398-1052)
run per world, one block each. The GPU equals the oracle's colour order bit
for bit: poses, velocities and the substep and impact counts.
"""
import numpy as np
import pytest

from nphysics_gb300 import abi, scenes
from oracle.oracle_py import ORDER_COLOUR, OracleWorld

pytestmark = pytest.mark.gpu


def make_pair(scene, params=None):
    from nphysics_gb300.world import GpuWorld
    p = params if params is not None else scene.params()
    g = GpuWorld.for_scene(scene, p)
    o = OracleWorld(p, scene.gravity, precision=32, order=ORDER_COLOUR)
    o.load_scene(scene)
    return g, o


def step_same(g, o, steps, per=1):
    subs = 0
    for _ in range(steps):
        g.step(per)
        o.step(per)
        gb, ob = g.bodies(), o.bodies()
        np.testing.assert_array_equal(gb["position"], ob["position"])
        np.testing.assert_array_equal(gb["velocity"], ob["velocity"])
        gc, oc = g.counters(), o.counters()
        assert (gc["ccd_substeps"], gc["ccd_impacts"]) == (oc["ccd_substeps"], oc["ccd_impacts"])
        subs += oc["ccd_substeps"]
    return subs


@pytest.mark.parametrize("shape,spin", [(abi.SHAPE_BALL, 0.0), (abi.SHAPE_CUBOID, 40.0), (abi.SHAPE_CAPSULE, 5.0)])
def test_projectiles_at_a_wall_match_oracle(gpu_lib, shape, spin):
    sc = scenes.ccd_wall(n=5, shape=shape, spin=spin)
    if shape == abi.SHAPE_CAPSULE:
        sc.colliders["shape_params"][1:] = (0.08, 0.15, 0.0)
    g, o = make_pair(sc)
    assert step_same(g, o, 6) >= 1
    assert (g.bodies()["position"][1:, 0] < -0.05).all()


@pytest.mark.parametrize("schedule", [abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS])
def test_struck_tower_matches_oracle(gpu_lib, schedule):
    sc = scenes.ccd_stack(height=4, balls=3)
    p = sc.params()
    p.solver_schedule = schedule
    g, o = make_pair(sc, p)
    assert step_same(g, o, 40) >= 1


def test_batched_ccd_worlds_match_oracle(gpu_lib):
    # Each world runs its own CCD loop: its own impacts, latest TOI and substeps.
    sc = scenes.batched_ccd(n_worlds=6)
    p = sc.params()
    p.solver_schedule = abi.SCHEDULE_WORLDS
    g, o = make_pair(sc, p)
    assert step_same(g, o, 30) >= 3


def test_ccd_batch_wider_than_the_gpu_matches_oracle(gpu_lib):
    # More CCD worlds than SMs: the pass kernel runs 128 threads a world
    # (256 for smaller batches); the results are the oracle's either way.
    sc = scenes.batched_ccd(n_worlds=160)
    p = sc.params()
    p.solver_schedule = abi.SCHEDULE_WORLDS
    g, o = make_pair(sc, p)
    assert step_same(g, o, 12) >= 12


def test_ccd_options_match_oracle(gpu_lib):
    # Four substeps, linear motion interpolation, the penetration switch.
    sc = scenes.ccd_wall(n=4, gravity=(0.0, -9.81, 0.0))
    p = sc.params()
    p.max_ccd_substeps = 4
    g, o = make_pair(sc, p)
    step_same(g, o, 10)
    sc = scenes.ccd_wall(n=4, shape=abi.SHAPE_CUBOID, spin=30.0, linear_interp=True)
    g, o = make_pair(sc)
    step_same(g, o, 8)
    sc = scenes.ccd_wall(n=2)
    sc.bodies["position"][1, 0] = -0.1
    p = sc.params()
    p.ccd_on_penetration_enabled = 1
    g, o = make_pair(sc, p)
    step_same(g, o, 3)


def test_ccd_with_graphs_and_removal(gpu_lib):
    # CCD steps replayed from a CUDA graph equal the eager steps; removing
    # the CCD colliders turns CCD off (the remaining bodies still match).
    sc = scenes.ccd_stack(height=3, balls=2)
    p = sc.params()
    p.use_graph = 1
    g, o = make_pair(sc, p)
    step_same(g, o, 20)
    for w in (g, o):
        w.remove_colliders(sc.collider_handles[-2:])
    step_same(g, o, 5)
    assert g.counters()["ccd_substeps"] == 0


def test_autotune_with_ccd_keeps_the_bits(gpu_lib):
    sc = scenes.batched_ccd(n_worlds=3)
    g, o = make_pair(sc)
    g.autotune(steps_per_candidate=2)
    g.step(5)
    o.step(int(g.counters()["steps"]))
    np.testing.assert_array_equal(g.bodies()["position"], o.bodies()["position"])
    np.testing.assert_array_equal(g.bodies()["velocity"], o.bodies()["velocity"])

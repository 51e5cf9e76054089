"""Joint constraints on the GPU against the oracle (through the C ABI).

Ball and fixed joints are solver manifolds of their own: coloured with the
contact manifolds, their bilateral rows solved with the friction rows, their
position rows with the contacts' (src/joint/ball_constraint.rs,
fixed_constraint.rs, solver/helper.rs:167-611, sor_prox.rs:232-293,
nonlinear_sor_prox.rs:57-117). The GPU equals the oracle's colour order bit
for bit: poses, velocities and the joints' cached impulses.
"""
import math

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


def assert_same(g, o, sc):
    gb, ob = g.bodies(), o.bodies()
    np.testing.assert_array_equal(gb["position"], ob["position"])
    np.testing.assert_array_equal(gb["velocity"], ob["velocity"])
    gi, gbk, gact = g.joints(sc.joint_handles)
    oi, obk, oact = o.joints(sc.joint_handles)
    np.testing.assert_array_equal(gi, oi.astype(np.float32))
    np.testing.assert_array_equal(gbk, obk)
    np.testing.assert_array_equal(gact, oact)


@pytest.mark.parametrize("sweep", [abi.SWEEP_SEPARATE, abi.SWEEP_MANIFOLD])
@pytest.mark.parametrize("graph", [0, 1])
def test_jointed_scene_matches_oracle_on_the_grid(gpu_lib, sweep, graph):
    sc = scenes.jointed()
    p = sc.params()
    p.solver_schedule = abi.SCHEDULE_GRID
    p.sweep_order = sweep
    p.use_graph = graph
    g, o = make_pair(sc, p)
    for _ in range(6):
        g.step(20)
        o.step(20)
        assert_same(g, o, sc)
    assert g.counters()["num_contacts"] > 20


@pytest.mark.parametrize("threads", [64, 256])
def test_batched_jointed_worlds_match_oracle(gpu_lib, threads):
    sc = scenes.batched_jointed(n_worlds=8)
    p = sc.params()
    p.solver_schedule = abi.SCHEDULE_WORLDS
    p.world_threads = threads
    g, o = make_pair(sc, p)
    for _ in range(4):
        g.step(30)
        o.step(30)
        assert_same(g, o, sc)


def test_jointed_worlds_sharded_step_to_the_same_bits(gpu_lib):
    # Joint priorities hash world-local joint slots: a shard of the batch
    # steps its worlds to the bits of the whole batch.
    from nphysics_gb300.world import GpuWorld
    whole = scenes.batched_jointed(n_worlds=6)
    part = scenes.batched_jointed(n_worlds=6, worlds=range(3, 6))
    gw, gp = GpuWorld.for_scene(whole), GpuWorld.for_scene(part)
    gw.step(60)
    gp.step(60)
    first = int(np.searchsorted(whole.bodies["world"], 3))
    np.testing.assert_array_equal(gw.bodies()["position"][first:], gp.bodies()["position"])


def test_pendulum_on_the_gpu(gpu_lib):
    # The oracle's pendulum KAT on the GPU: the period of a 2 m pendulum
    # released at 0.1 rad.
    from nphysics_gb300.world import GpuWorld
    sc = scenes.pendulum(length=2.0, angle=0.1)
    g = GpuWorld.for_scene(sc)
    xs = []
    for _ in range(600):
        g.step(1)
        xs.append(g.bodies()["position"][1, 0])
    crossings = [i for i in range(1, 600) if xs[i - 1] > 0 >= xs[i]]
    period = np.diff(crossings).mean() / 60.0
    expected = 2 * math.pi * math.sqrt(2.0 / 9.81) * (1 + 0.1 ** 2 / 16)
    assert abs(period - expected) < 0.004 * expected


def test_break_and_removal_match_oracle(gpu_lib):
    sc = scenes.jointed(chains=2, links=4, clusters=2, balls=0)
    sc.joints["break_force"][1] = 0.05       # a chain joint that gives way (the links below weigh 0.75 N)
    g, o = make_pair(sc)
    g.step(10)
    o.step(10)
    assert_same(g, o, sc)
    assert g.joints(sc.joint_handles)[1][1]
    # Remove a fixed joint and a chain's third link (body 3), and with it
    # joints 2 and 3, which hold it.
    for w in (g, o):
        w.remove_joints(sc.joint_handles[-1:])
        w.remove_bodies(sc.body_handles[3:4])
    g.step(40, joints=len(sc.joints) - 3)
    o.step(40)
    keep = np.ones(len(sc.joints), bool)
    keep[[-1, 2, 3]] = False
    gb, ob = g.bodies(), o.bodies()
    alive = np.ones(len(sc.bodies), bool)
    alive[3] = False
    np.testing.assert_array_equal(gb["position"][alive], ob["position"][alive])
    gi = g.joints(sc.joint_handles[keep])[0]
    oi = o.joints(sc.joint_handles[keep])[0]
    np.testing.assert_array_equal(gi, oi.astype(np.float32))


@pytest.mark.parametrize("sweep", [abi.SWEEP_SEPARATE, abi.SWEEP_MANIFOLD])
def test_every_joint_kind_matches_oracle(gpu_lib, sweep):
    # Ball, fixed, revolute, cartesian, planar, rectangular and universal
    # joints with contacts, on the one grid, and batched on the per-world
    # schedule.
    for sc, sched in ((scenes.joint_zoo(), abi.SCHEDULE_GRID), (scenes.batched_zoo(n_worlds=6), abi.SCHEDULE_WORLDS)):
        p = sc.params()
        p.solver_schedule = sched
        p.sweep_order = sweep
        g, o = make_pair(sc, p)
        for _ in range(4):
            g.step(40)
            o.step(40)
            assert_same(g, o, sc)


def test_hinge_pendulum_on_the_gpu(gpu_lib):
    # The oracle's revolute KAT on the GPU: the hinged box's period.
    from nphysics_gb300.world import GpuWorld
    a, b = 0.5, 0.1
    sc = scenes.hinge(kind=abi.JOINT_REVOLUTE, half=(a, b, 0.1), angle=math.pi / 2 - 0.15)
    g = GpuWorld.for_scene(sc)
    th = []
    for _ in range(600):
        g.step(1)
        q = g.bodies()["position"][1, 3:7]
        th.append(2.0 * math.atan2(q[2], q[3]) + math.pi / 2)
    crossings = [i for i in range(1, 600) if th[i - 1] > 0 >= th[i]]
    period = np.diff(crossings).mean() / 60.0
    ip = (a * a + b * b) / 3 + a * a
    expected = 2 * math.pi * math.sqrt(ip / (9.81 * a)) * (1 + 0.15 ** 2 / 16)
    assert abs(period - expected) < 0.01 * expected


def test_joint_errors_are_statuses(gpu_lib):
    from nphysics_gb300.world import GpuWorld, NpgpuError
    sc = scenes.batched_jointed(n_worlds=2)
    g = GpuWorld.for_scene(sc)
    with pytest.raises(NpgpuError) as e:
        g.step(1, joints=0)                  # the caller's set differs from the uploaded joints
    assert e.value.status == 4
    d = scenes.joint_descs(1)
    d["body1"]["index"], d["body2"]["index"] = 1, len(sc.bodies) - 1   # two worlds
    h = scenes.make_handles(1)
    h["index"] = 1000
    with pytest.raises(NpgpuError) as e:
        g.upsert_joints(h, d)
    assert e.value.status == abi_status("INVALID_ARGUMENT")
    d["body2"]["index"] = 1                  # the same body twice
    with pytest.raises(NpgpuError):
        g.upsert_joints(h, d)
    d["body2"]["index"] = 2
    d["body2"]["generation"] = 7             # a stale handle
    with pytest.raises(NpgpuError) as e:
        g.upsert_joints(h, d)
    assert e.value.status == abi_status("INVALID_HANDLE")
    bad = scenes.make_handles(1)
    bad["index"] = 999
    with pytest.raises(NpgpuError):
        g.joints(bad)
    g.step(2)                                # the world stays usable


def abi_status(name):
    return {"INVALID_HANDLE": 1, "INVALID_ARGUMENT": 10}[name]


def test_autotune_with_joints_keeps_the_bits(gpu_lib):
    # The tuner's steps carry the uploaded joints: the tuned jointed world
    # equals the oracle stepped as many times.
    sc = scenes.batched_zoo(n_worlds=4)
    g, o = make_pair(sc)
    sched, threads, ms = g.autotune(steps_per_candidate=2)
    assert ms > 0
    g.step(5)
    o.step(int(g.counters()["steps"]))
    gb, ob = g.bodies(), o.bodies()
    np.testing.assert_array_equal(gb["position"], ob["position"])
    np.testing.assert_array_equal(gb["velocity"], ob["velocity"])

"""Error behaviour of the C ABI on a GPU: statuses instead of aborts."""
import numpy as np
import pytest

from nphysics_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def world(**kw):
    from nphysics_gb300.world import GpuWorld
    return GpuWorld(**kw)


def test_rejects_unsupported_bodies_and_shapes(gpu_lib):
    from nphysics_gb300.world import NpgpuError
    w = world()
    b = scenes.body_descs(1)
    b["kind"] = abi.KIND_MULTIBODY
    with pytest.raises(NpgpuError) as e:
        w.upsert_bodies(scenes.make_handles(1), b)
    assert e.value.status == abi.ERR_UNSUPPORTED_BODY
    b["kind"] = abi.KIND_RIGID_BODY
    w.upsert_bodies(scenes.make_handles(1), b)
    c = scenes.collider_descs(1, 0, abi.SHAPE_OTHER, (1, 1, 1), density=1.0)
    with pytest.raises(NpgpuError) as e:
        w.upsert_colliders(scenes.make_handles(1), c)
    assert e.value.status == abi.ERR_UNSUPPORTED_SHAPE


def test_rejects_joints_and_force_generators(gpu_lib):
    from nphysics_gb300.world import NpgpuError
    w = world()
    with pytest.raises(NpgpuError) as e:
        w.step(1, joints=1)
    assert e.value.status == abi.ERR_NONEMPTY_JOINTS
    with pytest.raises(NpgpuError) as e:
        w.step(1, force_generators=2)
    assert e.value.status == abi.ERR_NONEMPTY_FORCES


def test_invalid_handles_and_nan(gpu_lib):
    from nphysics_gb300.world import NpgpuError
    w = world()
    b = scenes.body_descs(2)
    w.upsert_bodies(scenes.make_handles(2), b)
    stale = scenes.make_handles(1, generation=7)
    with pytest.raises(NpgpuError) as e:
        w.remove_bodies(stale)
    assert e.value.status == abi.ERR_INVALID_HANDLE
    c = scenes.collider_descs(1, 0, abi.SHAPE_BALL, (0.5, 0, 0), density=1.0)
    c["body"]["generation"] = 3
    with pytest.raises(NpgpuError) as e:
        w.upsert_colliders(scenes.make_handles(1), c)
    assert e.value.status == abi.ERR_INVALID_HANDLE
    b["position"][0, 0] = np.nan
    with pytest.raises(NpgpuError) as e:
        w.upsert_bodies(scenes.make_handles(2), b)
    assert e.value.status == abi.ERR_NAN


def test_pair_capacity_overflow_is_reported(gpu_lib):
    from nphysics_gb300.world import GpuWorld, NpgpuError
    sc = scenes.ball_pile(side=4, spacing=1.0)
    w = GpuWorld(sc.params(), sc.gravity, capacity_bodies=len(sc.bodies), capacity_colliders=len(sc.colliders),
                 capacity_pairs=8)
    w.load_scene(sc)
    with pytest.raises(NpgpuError) as e:
        w.step(1)
    assert e.value.status == abi.ERR_CAPACITY
    # The world stays usable: the error is cleared after it was reported.
    w.synchronize()


def test_capacity_of_slots(gpu_lib):
    from nphysics_gb300.world import NpgpuError
    w = world(capacity_bodies=4, capacity_colliders=4)
    h = scenes.make_handles(5)
    with pytest.raises(NpgpuError) as e:
        w.upsert_bodies(h, scenes.body_descs(5))
    assert e.value.status == abi.ERR_CAPACITY


def platform_scene(side):
    """side x side balls resting on one dynamic platform on the ground: the
    platform takes part in side^2 + 1 solver manifolds, so it needs as many
    colours."""
    g, gc = scenes._ground()
    plat = scenes.body_descs(1)
    plat["position"][0, :3] = (0.0, 0.5, 0.0)
    pc = scenes.collider_descs(1, 0, abi.SHAPE_CUBOID, (6.0, 0.5, 6.0), density=1.0)
    n = side * side
    b = scenes.body_descs(n)
    i = np.arange(n)
    b["position"][:, 0] = (i % side - (side - 1) / 2) * 1.05
    b["position"][:, 1] = 1.49
    b["position"][:, 2] = (i // side - (side - 1) / 2) * 1.05
    bc = scenes.collider_descs(n, np.arange(n), abi.SHAPE_BALL, (0.5, 0, 0), density=1.0)
    return scenes.Scene("platform", *scenes._concat([g, plat, b], [gc, pc, bc]))


@pytest.mark.parametrize("sched", [abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS])
def test_more_than_56_colours_match_the_oracle(gpu_lib, sched):
    # 64 balls on the platform: 65 colours, past one colour word; the second
    # word carries colours 56-111 and the bits still match the oracle.
    from nphysics_gb300.world import GpuWorld
    from oracle.oracle_py import ORDER_COLOUR, OracleWorld
    sc = platform_scene(8)
    p = sc.params()
    p.solver_schedule = sched
    g = GpuWorld.for_scene(sc, p)
    o = OracleWorld(p, sc.gravity, precision=32, order=ORDER_COLOUR)
    o.load_scene(sc)
    g.step(5)
    o.step(5)
    assert g.counters()["num_colours"] > 56
    gb, ob = g.bodies(), o.bodies()
    np.testing.assert_array_equal(gb["position"], ob["position"])
    np.testing.assert_array_equal(gb["velocity"], ob["velocity"])


@pytest.mark.parametrize("sched", [abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS])
def test_too_many_colours_is_reported(gpu_lib, sched):
    # 121 balls give the platform 122 solver manifolds, more than the 112
    # colours a step can use: the step reports a capacity error (the solver
    # kernels stand down at once rather than wait on an inconsistent order),
    # and the world stays usable.
    import time
    from nphysics_gb300.world import GpuWorld, NpgpuError
    sc = platform_scene(11)
    p = sc.params()
    p.solver_schedule = sched
    w = GpuWorld.for_scene(sc, p)
    t0 = time.perf_counter()
    with pytest.raises(NpgpuError) as e:
        w.step(1)
    assert e.value.status == abi.ERR_CAPACITY
    assert "colours" in str(e.value)
    assert time.perf_counter() - t0 < 0.9          # no bounded wait ran out
    w.synchronize()

"""Parity of the GPU step with the oracle (colour order, f32) on the parts of
the reference's path that the piles and stacks leave out: kinematic bodies,
locked degrees of freedom, restitution and material combine modes, damping
and velocity clamps, bodies with several colliders, applied forces, and
sleep. Every comparison is bit for bit: both sides evaluate the same
operations in the same order without fused multiply-add."""
import numpy as np
import pytest

from nphysics_gb300 import abi, scenes
from oracle.oracle_py import ORDER_COLOUR, OracleWorld

pytestmark = pytest.mark.gpu


def pair(scene, params=None):
    from nphysics_gb300.world import GpuWorld
    p = params if params is not None else scene.params()
    g = GpuWorld.for_scene(scene, p)
    o = OracleWorld(p, scene.gravity, precision=32, order=ORDER_COLOUR)
    o.load_scene(scene)
    return g, o


def same(g, o, what=""):
    gb, ob = g.bodies(), o.bodies()
    for k in ("position", "velocity"):
        np.testing.assert_array_equal(gb[k], ob[k], err_msg=f"{what}: {k}")
    np.testing.assert_array_equal(gb["active"], ob["active"], err_msg=f"{what}: active")


def balls_on_ground(n=12, seed=0, spacing=1.05):
    rng = np.random.default_rng(seed)
    g, gc = scenes._ground()
    b = scenes.body_descs(n)
    side = int(np.ceil(np.sqrt(n)))
    idx = np.arange(n)
    b["position"][:, 0] = (idx % side) * spacing + rng.uniform(-0.02, 0.02, n)
    b["position"][:, 1] = 0.52 + (idx // (side * side)) * 1.0
    b["position"][:, 2] = (idx // side % side) * spacing + rng.uniform(-0.02, 0.02, n)
    c = scenes.collider_descs(n, np.arange(n), abi.SHAPE_BALL, (0.5, 0, 0), density=1.0, friction=0.5)
    return [g, b], [gc, c]


def test_kinematic_body_pushes_dynamic_ones(gpu_lib):
    pb, pc = balls_on_ground(12)
    k = scenes.body_descs(1)
    k["status"] = abi.BODY_KINEMATIC
    k["position"][0, :3] = (-2.0, 0.6, 1.0)
    k["velocity"][0, :3] = (2.0, 0.0, 0.0)
    k["velocity"][0, 3:] = (0.0, 0.5, 0.0)
    kc = scenes.collider_descs(1, 0, abi.SHAPE_CUBOID, (0.5, 0.5, 1.5), density=1.0)
    bodies, colliders = scenes._concat(pb + [k], pc + [kc])
    sc = scenes.Scene("kinematic plough", bodies, colliders)
    g, o = pair(sc)
    g.step(90)
    o.step(90)
    same(g, o, "kinematic")
    moved = np.abs(g.bodies()["position"][1:13, 0] - sc.bodies["position"][1:13, 0]).max()
    assert moved > 0.1


def test_locked_degrees_of_freedom(gpu_lib):
    sc = scenes.random_cluster(n=24, seed=12, extent=2.0)
    locks = [abi.BODY_LOCK_RX | abi.BODY_LOCK_RY | abi.BODY_LOCK_RZ, abi.BODY_LOCK_TX | abi.BODY_LOCK_TZ,
             abi.BODY_LOCK_RY, abi.BODY_LOCK_TY | abi.BODY_LOCK_RX]
    dyn = np.nonzero(sc.bodies["status"] == abi.BODY_DYNAMIC)[0]
    for i, b in enumerate(dyn):
        sc.bodies["flags"][b] |= locks[i % len(locks)]
    # A lock masks forces and impulses; a body keeps the velocity it was
    # given (jacobian_mask, rigid_body.rs:708), so the rotation-locked ones
    # start without spin.
    rot_locked = dyn[0::len(locks)]
    sc.bodies["velocity"][rot_locked, 3:] = 0.0
    g, o = pair(sc)
    g.step(80)
    o.step(80)
    same(g, o, "locks")
    # Bodies with every rotation locked kept their orientation.
    np.testing.assert_allclose(g.bodies()["position"][rot_locked, 3:7], sc.bodies["position"][rot_locked, 3:7],
                               rtol=0, atol=1e-6)


def test_restitution_and_combine_modes(gpu_lib):
    pb, pc = balls_on_ground(16, seed=3, spacing=1.3)
    pb[1]["position"][:, 1] += 3.0
    c = pc[1]
    c["restitution"] = np.linspace(0.0, 0.9, len(c)).astype(np.float32)
    c["friction"] = np.linspace(0.1, 1.0, len(c)).astype(np.float32)
    modes = [abi.COMBINE_AVERAGE, abi.COMBINE_MIN, abi.COMBINE_MULTIPLY, abi.COMBINE_MAX]
    c["friction_combine"] = [modes[i % 4] for i in range(len(c))]
    c["restitution_combine"] = [modes[(i + 1) % 4] for i in range(len(c))]
    pc[0]["restitution"] = 0.5
    bodies, colliders = scenes._concat(pb, pc)
    sc = scenes.Scene("bouncing balls", bodies, colliders)
    g, o = pair(sc)
    g.step(150)
    o.step(150)
    same(g, o, "restitution")


def test_damping_and_velocity_clamps(gpu_lib):
    sc = scenes.random_cluster(n=30, seed=21, extent=2.5)
    dyn = sc.bodies["status"] == abi.BODY_DYNAMIC
    sc.bodies["velocity"][dyn] *= 8.0
    sc.bodies["linear_damping"][dyn] = np.linspace(0.0, 2.0, int(dyn.sum()))
    sc.bodies["angular_damping"][dyn] = np.linspace(1.0, 0.0, int(dyn.sum()))
    sc.bodies["max_linear_velocity"][dyn] = np.where(np.arange(int(dyn.sum())) % 2 == 0, 3.0, abi.FLT_MAX)
    sc.bodies["max_angular_velocity"][dyn] = np.where(np.arange(int(dyn.sum())) % 3 == 0, 2.0, abi.FLT_MAX)
    g, o = pair(sc)
    g.step(60)
    o.step(60)
    same(g, o, "damping")


def test_bodies_with_several_colliders(gpu_lib):
    # Dumbbells (two offset balls) and boxes with an offset, rotated collider.
    g0, gc0 = scenes._ground()
    n = 8
    b = scenes.body_descs(n)
    b["position"][:, 0] = np.arange(n) * 2.5 - 8.0
    b["position"][:, 1] = 2.0 + 0.3 * np.arange(n)
    b["position"][:, 3:7] = scenes.uniform_quaternions(np.random.default_rng(5), n)
    parts_c = []
    for i in range(n):
        if i % 2 == 0:
            c = scenes.collider_descs(2, i, abi.SHAPE_BALL, (0.4, 0, 0), density=1.0)
            c["position_wrt_body"][0, :3] = (-0.6, 0.0, 0.0)
            c["position_wrt_body"][1, :3] = (0.6, 0.1, 0.0)
            c["density"][1] = 3.0
        else:
            c = scenes.collider_descs(2, i, abi.SHAPE_CUBOID, (0.3, 0.2, 0.5), density=1.0)
            c["position_wrt_body"][1, :3] = (0.0, 0.5, 0.2)
            c["position_wrt_body"][1, 3:7] = (0.0, 0.3826834, 0.0, 0.9238795)
        parts_c.append(c)
    colliders = np.concatenate(parts_c)
    bodies, colliders = scenes._concat([g0, b], [gc0, colliders])
    sc = scenes.Scene("compound bodies", bodies, colliders)
    g, o = pair(sc)
    g.step(1)
    o.step(1)
    gi, gc = g.mass_properties()
    oi, oc = o.mass_properties()
    np.testing.assert_array_equal(gi, oi)
    np.testing.assert_array_equal(gc, oc)
    g.step(100)
    o.step(100)
    same(g, o, "compound")


def test_applied_forces_and_sleep(gpu_lib):
    pb, pc = balls_on_ground(9, seed=8)
    bodies, colliders = scenes._concat(pb, pc)
    sc = scenes.Scene("forces", bodies, colliders)
    g, o = pair(sc)
    g.step(240)
    o.step(240)
    same(g, o, "settled")
    assert g.bodies()["active"][1:].sum() == 0          # all asleep
    h = np.ascontiguousarray(sc.body_handles[[1, 4, 7]])
    f = np.zeros((3, 6), np.float32)
    f[:, 0] = (30.0, -20.0, 5.0)
    f[:, 4] = (3.0, 0.0, -2.0)
    for k in range(20):
        g.apply_forces(h, f, wake=(k == 0))
        o.apply_forces(h, f, wake=(k == 0))
        g.step(1)
        o.step(1)
    same(g, o, "pushed")
    assert g.bodies()["active"][[1, 4, 7]].all()


def test_pinned_host_buffers(gpu_lib):
    # Forces read from and poses written to page-locked host arrays (the
    # copy engines reach them directly) give what pageable arrays give; a
    # force batch with one bad handle is rejected whole.
    import torch

    def pinned(a):
        buf = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True).numpy()
        out = buf.view(a.dtype).reshape(a.shape)
        out[...] = a
        return out

    pb, pc = balls_on_ground(9, seed=3)
    bodies, colliders = scenes._concat(pb, pc)
    sc = scenes.Scene("pinned", bodies, colliders)
    g, o = pair(sc)
    h = np.ascontiguousarray(sc.body_handles[[2, 5]])
    f = np.zeros((2, 6), np.float32)
    f[:, 1] = (40.0, 25.0)
    hp, fp = pinned(h), pinned(f)
    bad = h.copy()
    bad[1]["generation"] += 1
    from nphysics_gb300.world import NpgpuError
    with pytest.raises(NpgpuError) as e:
        g.apply_forces(pinned(bad), fp)
    assert e.value.status == abi.ERR_INVALID_HANDLE
    for _ in range(30):
        g.apply_forces(hp, fp, wake=True)
        o.apply_forces(h, f, wake=True)
        g.step(1)
        o.step(1)
    same(g, o, "pinned forces")
    n = g.num_bodies
    pos, vel = pinned(np.zeros((n, 7), np.float32)), pinned(np.zeros((n, 6), np.float32))
    g.download_into(pos, vel)
    ref = g.bodies()
    np.testing.assert_array_equal(pos, ref["position"])
    np.testing.assert_array_equal(vel, ref["velocity"])


def test_forces_naming_a_body_twice(gpu_lib):
    # A batch that names one body twice adds both forces in the batch's order,
    # as the reference's successive apply_force calls do.
    pb, pc = balls_on_ground(9, seed=4)
    bodies, colliders = scenes._concat(pb, pc)
    sc = scenes.Scene("twice", bodies, colliders)
    g, o = pair(sc)
    h = np.ascontiguousarray(sc.body_handles[[3, 6, 3, 3]])
    f = np.zeros((4, 6), np.float32)
    f[:, 0] = (0.1, 5.0, 1e-3, 7.0)
    f[:, 4] = (1e-4, -2.0, 3.0, 0.3)
    for _ in range(10):
        g.apply_forces(h, f, wake=True)
        o.apply_forces(h, f, wake=True)
        g.step(1)
        o.step(1)
    same(g, o, "twice")

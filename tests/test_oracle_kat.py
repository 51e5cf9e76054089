"""Known-answer tests of the CPU oracle (no GPU).

The reference's own test of this path is the cuboid mass-properties check of
src/volumetric/volumetric_convex3.rs:285-346 (a 0.96 half-extent cube, density
2.37689, epsilon 1e-8). The rest are analytic checks of the restated step:
free fall under the semi-implicit Euler step, friction deceleration, resting
contact impulses and sleeping.
"""
import math

import numpy as np
import pytest

from nphysics_gb300 import abi, scenes
from oracle.oracle_py import ORDER_COLOUR, ORDER_REFERENCE, OracleWorld


def _convex_box_mass_properties(half, shift, density):
    """Mass, COM and inertia of a triangulated box by signed tetrahedra (the
    method a convex-hull volumetric uses), independent of the cuboid formula."""
    hx, hy, hz = half
    v = np.array([[sx * hx, sy * hy, sz * hz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)]) + shift
    # 12 outward-facing triangles of the box (vertex index = 4 sx + 2 sy + sz).
    faces = [(0, 1, 3), (0, 3, 2), (4, 6, 7), (4, 7, 5), (0, 4, 5), (0, 5, 1), (2, 3, 7), (2, 7, 6),
             (0, 2, 6), (0, 6, 4), (1, 5, 7), (1, 7, 3)]
    vol = 0.0
    com = np.zeros(3)
    cov = np.zeros((3, 3))
    canon = np.array([[2, 1, 1], [1, 2, 1], [1, 1, 2]]) / 120.0
    for a, b, c in faces:
        A = np.stack([v[a], v[b], v[c]], axis=1)
        d = np.linalg.det(A)
        vol += d / 6.0
        com += d / 6.0 * (v[a] + v[b] + v[c]) / 4.0
        cov += d * A @ canon @ A.T
    com /= vol
    cov = density * cov
    mass = density * vol
    cov -= mass * np.outer(com, com)
    inertia = np.trace(cov) * np.eye(3) - cov
    return mass, com, inertia


def test_cuboid_mass_properties_match_reference_kat():
    # volumetric_convex3.rs:292-345: the convex hull of a shifted 2 - 0.08 wide
    # cube matches Cuboid(0.96) unit inertia and mass_properties(2.37689), eps 1e-8.
    # The descriptors carry f32; the KAT uses the same f32-rounded inputs.
    h32 = float(np.float32(0.96))
    half = (h32, h32, h32)
    density = float(np.float32(2.37689))
    m_hull, _, i_hull = _convex_box_mass_properties(half, np.array([10.0, 10.0, 10.0]), density)
    sc = scenes.single_body(shape=abi.SHAPE_CUBOID, params=half, ground=False, density=density)
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(1)
    inertia, com = w.mass_properties()
    assert abs(inertia[0, 0] - m_hull) < 1e-8 * max(1.0, m_hull)
    expected = [i_hull[0, 0], i_hull[0, 1], i_hull[0, 2], i_hull[1, 1], i_hull[1, 2], i_hull[2, 2]]
    np.testing.assert_allclose(inertia[0, 1:], expected, rtol=0, atol=1e-8 * m_hull)
    # Unit inertia (4/12)(hy^2 + hz^2) = 0.6144 for 0.96 (f32-rounded input).
    assert abs(inertia[0, 1] / inertia[0, 0] - (4.0 / 12.0) * 2 * h32 * h32) < 1e-12
    np.testing.assert_allclose(com[0], 0.0, atol=1e-15)


def test_ball_mass_properties():
    r, density = float(np.float32(0.7)), 3.0
    sc = scenes.single_body(shape=abi.SHAPE_BALL, params=(r, 0, 0), ground=False, density=density)
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(1)
    inertia, _ = w.mass_properties()
    m = 4.0 / 3.0 * math.pi * r ** 3 * density
    assert abs(inertia[0, 0] - m) < 1e-12 * m
    assert abs(inertia[0, 1] - 0.4 * m * r * r) < 1e-12 * m


@pytest.mark.parametrize("precision", [32, 64])
def test_free_fall_is_semi_implicit_euler(precision):
    sc = scenes.single_body(shape=abi.SHAPE_BALL, params=(0.5, 0, 0), position=(0, 100, 0), ground=False)
    w = OracleWorld(sc.params(), sc.gravity, precision=precision)
    w.load_scene(sc)
    dt, g = float(np.float32(1.0 / 60.0)), float(np.float32(-9.81))   # the parameters travel as f32
    n = 60
    w.step(n)
    b = w.bodies()
    v = g * dt * n
    y = 100.0 + g * dt * dt * n * (n + 1) / 2.0
    tol = 1e-9 if precision == 64 else 2e-4
    assert abs(b["velocity"][0, 1] - v) < tol * 10
    assert abs(b["position"][0, 1] - y) < tol * 100


def test_torque_free_spin_keeps_angular_momentum_direction():
    # Gyroscopic term (rigid_body.rs:575-581, 598-605) on an asymmetric box spinning about a
    # near-principal axis: |L| stays nearly constant over a second.
    sc = scenes.single_body(shape=abi.SHAPE_CUBOID, params=(0.2, 0.5, 1.0), position=(0, 100, 0),
                            velocity=(0, 0, 0, 5.0, 0.1, 0.1), ground=False)
    sc.bodies["flags"] = sc.bodies["flags"] & np.uint32(0xffffffff ^ abi.BODY_GRAVITY)
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(1)

    def ang_momentum():
        b = w.bodies()
        q = b["position"][0, 3:7]
        x, y, z, ww = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * ww), 2 * (x * z + y * ww)],
                      [2 * (x * y + z * ww), 1 - 2 * (x * x + z * z), 2 * (y * z - x * ww)],
                      [2 * (x * z - y * ww), 2 * (y * z + x * ww), 1 - 2 * (x * x + y * y)]])
        inertia, _ = w.mass_properties()
        I = np.diag([inertia[0, 1], inertia[0, 4], inertia[0, 6]])
        return R @ I @ R.T @ b["velocity"][0, 3:]

    L0 = ang_momentum()
    w.step(60)
    L1 = ang_momentum()
    assert np.linalg.norm(L1 - L0) < 0.02 * np.linalg.norm(L0)


def test_resting_box_normal_impulse_balances_gravity():
    sc = scenes.single_body(shape=abi.SHAPE_CUBOID, params=(0.5, 0.5, 0.5), position=(0, 0.5, 0))
    p = sc.params()
    p.solve_to_tolerance = 1
    p.residual_tolerance = 1e-7
    p.max_iterations_to_tolerance = 500
    w = OracleWorld(p, sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(30)
    c = w.contacts_f64()
    m = 1.0   # 1 x 1 x 1 box, density 1
    total = c[:, 10].sum()
    assert abs(total - m * 9.81 / 60.0) < 1e-6
    b = w.bodies()
    # Rests with the margins overlapping by the allowed linear error (0.001).
    assert abs(b["position"][1, 1] - (0.5 + 0.02 - 0.001)) < 2e-4


def test_friction_stops_a_sliding_box_at_mu_g():
    sc = scenes.single_body(shape=abi.SHAPE_CUBOID, params=(0.5, 0.5, 0.5), position=(0, 0.5, 0),
                            velocity=(1.0, 0, 0, 0, 0, 0))
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(5)
    v5 = w.bodies()["velocity"][1, 0]
    w.step(1)
    v6 = w.bodies()["velocity"][1, 0]
    decel = (v5 - v6) * 60.0
    assert abs(decel - 0.5 * 9.81) < 0.05 * 0.5 * 9.81
    w.step(30)
    assert abs(w.bodies()["velocity"][1, 0]) < 1e-6


def test_resting_body_falls_asleep_and_zeroes_velocity():
    sc = scenes.single_body(shape=abi.SHAPE_BALL, params=(0.5, 0, 0), position=(0, 0.5, 0))
    w = OracleWorld(sc.params(), sc.gravity, precision=32)
    w.load_scene(sc)
    w.step(400)
    b = w.bodies()
    assert b["active"][1] == 0
    assert np.all(b["velocity"][1] == 0)
    assert w.counters()["num_active_bodies"] == 0


def test_orders_converge_to_the_same_velocities():
    # The colour order is a permutation of the reference's Gauss-Seidel order,
    # and the per-manifold sweep order (each manifold's friction rows, then its
    # normal rows) another; run to a tight residual they all converge to the
    # same post-solve velocities.
    sc = scenes.pyramid(base=6)
    out = []
    for order, sweep in ((ORDER_REFERENCE, abi.SWEEP_SEPARATE), (ORDER_COLOUR, abi.SWEEP_SEPARATE),
                         (ORDER_COLOUR, abi.SWEEP_MANIFOLD)):
        p = sc.params()
        p.solve_to_tolerance = 1
        p.residual_tolerance = 1e-9
        p.max_iterations_to_tolerance = 5000
        p.max_position_iterations = 0
        p.sweep_order = sweep
        w = OracleWorld(p, sc.gravity, precision=64, order=order)
        w.load_scene(sc)
        w.step(1)
        out.append(w.bodies()["velocity"])
        assert w.counters()["residual"] <= 1e-9
    np.testing.assert_allclose(out[0], out[1], atol=1e-6)
    np.testing.assert_allclose(out[0], out[2], atol=1e-6)


def test_sweep_and_prune_equals_brute_force():
    sc = scenes.random_cluster(n=300, seed=3, extent=4.0)
    w = OracleWorld(sc.params(), sc.gravity, precision=32)
    w.load_scene(sc)
    w.step(3)
    w.collision_detection()
    a = w.pairs()
    b = w.brute_force_pairs()
    assert len(a) > 100
    np.testing.assert_array_equal(a, b)


def _no_gravity(sc):
    sc.bodies["flags"] = sc.bodies["flags"] & np.uint32(0xffffffff ^ abi.BODY_GRAVITY)
    return sc


F32_DT = float(np.float32(1.0 / 60.0))
F32_G = float(np.float32(9.81))


def test_damping_follows_the_integrate_recurrence():
    # RigidBody::integrate (rigid_body.rs:467-469, 503-504): each step v *= 1 / (1 + dt d),
    # then the pose moves by v dt. A free ball without gravity: nothing else acts on it.
    sc = _no_gravity(scenes.single_body(shape=abi.SHAPE_BALL, params=(0.5, 0, 0), position=(0, 100, 0),
                                        velocity=(3.0, 0, 0, 0, 0, 2.0), ground=False))
    sc.bodies["linear_damping"] = 0.5
    sc.bodies["angular_damping"] = 0.25
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    n = 30
    w.step(n)
    v, x, om, th = 3.0, 0.0, 2.0, 0.0
    for _ in range(n):
        v *= 1.0 / (1.0 + F32_DT * 0.5)
        om *= 1.0 / (1.0 + F32_DT * 0.25)
        x += v * F32_DT
        th += om * F32_DT
    b = w.bodies()
    assert abs(b["velocity"][0, 0] - v) < 1e-12
    assert abs(b["velocity"][0, 5] - om) < 1e-12
    assert abs(b["position"][0, 0] - x) < 1e-12
    q = b["position"][0, 3:7]            # (i, j, k, w): a rotation by th about z
    assert abs(abs(q[2]) - math.sin(th / 2)) < 1e-9 and abs(abs(q[3]) - math.cos(th / 2)) < 1e-9
    assert abs(q[0]) < 1e-12 and abs(q[1]) < 1e-12


@pytest.mark.parametrize("max_lin,max_ang", [(2.0, 1.0), (0.0, 0.0), (10.0, 10.0)])
def test_velocity_clamps_scale_to_the_maximum(max_lin, max_ang):
    # rigid_body.rs:471-501: a velocity whose norm is above the maximum is scaled to it; a zero
    # maximum zeroes it; below the maximum nothing changes.
    sc = _no_gravity(scenes.single_body(shape=abi.SHAPE_BALL, params=(0.5, 0, 0), position=(0, 100, 0),
                                        velocity=(3.0, 4.0, 0, 0, 0, 5.0), ground=False))
    sc.bodies["max_linear_velocity"] = max_lin
    sc.bodies["max_angular_velocity"] = max_ang
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(1)
    b = w.bodies()
    lin = np.array([3.0, 4.0, 0.0]) * min(1.0, max_lin / 5.0)
    ang = np.array([0.0, 0.0, 5.0]) * min(1.0, max_ang / 5.0)
    np.testing.assert_allclose(b["velocity"][0, :3], lin, atol=1e-12)
    np.testing.assert_allclose(b["velocity"][0, 3:], ang, atol=1e-12)
    np.testing.assert_allclose(b["position"][0, :3], np.array([0.0, 100.0, 0.0]) + lin * F32_DT, atol=1e-12)


def test_kinematic_body_keeps_its_velocity_through_contacts():
    # A kinematic box pushes a dynamic ball along the ground: gravity and the contact leave the
    # kinematic body's velocity alone, its pose advances by v dt each step, and the ball is pushed.
    parts_b, parts_c = [], []
    g, gc = scenes._ground()
    kb = scenes.body_descs(1)
    kb["status"] = abi.BODY_KINEMATIC
    kb["position"][0, :3] = (0.0, 0.5, 0.0)
    kb["velocity"][0, :3] = (1.0, 0.0, 0.0)
    kc = scenes.collider_descs(1, 0, abi.SHAPE_CUBOID, (0.5, 0.5, 0.5), density=1.0)
    bb = scenes.body_descs(1)
    bb["position"][0, :3] = (1.6, 0.5, 0.0)
    bc = scenes.collider_descs(1, 0, abi.SHAPE_BALL, (0.5, 0, 0), density=1.0)
    bodies, colliders = scenes._concat([g, kb, bb], [gc, kc, bc])
    sc = scenes.Scene("kinematic pusher", bodies, colliders)
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    n = 90
    w.step(n)
    x = 0.0
    for _ in range(n):
        x += 1.0 * F32_DT
    b = w.bodies()
    np.testing.assert_array_equal(b["velocity"][1], [1.0, 0, 0, 0, 0, 0])
    assert abs(b["position"][1, 0] - x) < 1e-12 and b["position"][1, 1] == np.float32(0.5)
    assert b["position"][2, 0] > 1.6 + 0.3          # the ball was pushed ahead of the box
    assert b["position"][2, 0] >= b["position"][1, 0] + 1.0 - 0.02 - 1e-3


def test_locked_translation_axis_does_not_move():
    # update_acceleration / the velocity update mask by jacobian_mask (rigid_body.rs:590-619):
    # with Y locked gravity does not move the body; the free X axis keeps its velocity.
    sc = scenes.single_body(shape=abi.SHAPE_BALL, params=(0.5, 0, 0), position=(0, 5, 0),
                            velocity=(1.0, 0, 0, 0, 0, 0))
    sc.bodies["flags"][1] |= np.uint32(abi.BODY_LOCK_TY)
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    n = 60
    w.step(n)
    x = 0.0
    for _ in range(n):
        x += 1.0 * F32_DT
    b = w.bodies()
    assert b["position"][1, 1] == 5.0 and b["velocity"][1, 1] == 0.0
    assert abs(b["position"][1, 0] - x) < 1e-12 and b["velocity"][1, 0] == 1.0


A, MN, MU, MX = abi.COMBINE_AVERAGE, abi.COMBINE_MIN, abi.COMBINE_MULTIPLY, abi.COMBINE_MAX


def _combine(a, b):
    """MaterialCombineMode::combine (material.rs:66-87): the mode of higher precedence wins."""
    modes = (a[1], b[1])
    if MX in modes:
        return max(a[0], b[0])
    if MU in modes:
        return a[0] * b[0]
    if MN in modes:
        return min(a[0], b[0])
    return (a[0] + b[0]) * 0.5


@pytest.mark.parametrize("speed,e_ball,m_ball,e_ground,m_ground,e", [
    (5.0, 1.0, A, 1.0, A, 1.0),
    (5.0, 1.0, A, 0.0, A, 0.5),      # Average
    (5.0, 0.8, MX, 0.2, A, 0.8),     # Max over Average
    (5.0, 0.8, MU, 0.5, MN, 0.4),    # Multiply over Min
    (5.0, 0.8, MN, 0.2, A, 0.2),     # Min over Average
    (5.0, 0.2, A, 0.8, MX, 0.8),     # either side's mode counts
    (0.5, 1.0, A, 1.0, A, 1.0),      # below restitution_velocity_threshold: no bounce (vy = 0)
])
def test_restitution_and_its_combine_rule(speed, e_ball, m_ball, e_ground, m_ground, e):
    # signorini_model.rs:94-97: if rhs <= -threshold then rhs += e rhs, e combined by
    # MaterialCombineMode::combine (material.rs:66-87: Max > Multiply > Min > Average). A ball
    # touching the ground (gap = the two margins, so no speculative term) hits it at `speed`;
    # solved to convergence, it leaves at e times its approach speed, gravity's dt g included.
    sc = scenes.single_body(shape=abi.SHAPE_BALL, params=(0.5, 0, 0), position=(0, 0.52, 0),
                            velocity=(0, -speed, 0, 0, 0, 0))
    c = sc.colliders
    c["restitution"][1], c["restitution_combine"][1] = e_ball, m_ball
    c["restitution"][0], c["restitution_combine"][0] = e_ground, m_ground
    p = sc.params()
    p.solve_to_tolerance = 1
    p.residual_tolerance = 1e-12
    p.max_iterations_to_tolerance = 200
    w = OracleWorld(p, sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(1)
    vy = w.bodies()["velocity"][1, 1]
    approach = speed + F32_G * F32_DT
    # The descriptors carry f32: combine the f32-rounded coefficients.
    ec = _combine((float(np.float32(e_ball)), m_ball), (float(np.float32(e_ground)), m_ground))
    assert abs(ec - e) < 1e-7
    if speed + F32_G * F32_DT < 1.0:
        ec = 0.0
    assert abs(vy - ec * approach) < 1e-9, (vy, ec * approach)


@pytest.mark.parametrize("mu_box,m_box,mu_ground,m_ground,mu", [
    (0.2, MU, 0.6, A, 0.12),
    (0.2, A, 0.6, MN, 0.2),
    (0.2, MX, 0.6, A, 0.6),
    (0.2, A, 0.6, A, 0.4),
])
def test_friction_combine_rule_sets_the_deceleration(mu_box, m_box, mu_ground, m_ground, mu):
    sc = scenes.single_body(shape=abi.SHAPE_CUBOID, params=(0.5, 0.5, 0.5), position=(0, 0.5, 0),
                            velocity=(3.0, 0, 0, 0, 0, 0))
    c = sc.colliders
    c["friction"][1], c["friction_combine"][1] = mu_box, m_box
    c["friction"][0], c["friction_combine"][0] = mu_ground, m_ground
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(5)
    v5 = w.bodies()["velocity"][1, 0]
    w.step(1)
    v6 = w.bodies()["velocity"][1, 0]
    decel = (v5 - v6) / F32_DT
    assert abs(decel - mu * F32_G) < 0.05 * mu * F32_G, (decel, mu * F32_G)


@pytest.mark.parametrize("k", [1, 2, 5])
def test_converged_stack_impulses_f32_colour_vs_f64(k):
    # The oracle's own f32 colour order (the GPU's sequence) solved to 1e-6
    # against its f64 build in the reference's order solved to 1e-12: the
    # converged normal impulses of a ball stack agree within 1e-4 relative
    # and equal the statics, i ball weights m g dt at the i-th contact from
    # the top.
    from nphysics_gb300 import abi as _abi
    g, gc = scenes._ground(friction=0.5)
    b = scenes.body_descs(k)
    b["position"][:, 1] = 0.5 + np.arange(k)
    c = scenes.collider_descs(k, np.arange(k), _abi.SHAPE_BALL, (0.5, 0, 0), density=1.0, friction=0.5)
    bodies, colliders = scenes._concat([g, b], [gc, c])
    sc = scenes.Scene("ball stack", bodies, colliders)
    out = []
    for prec, order, tol in ((32, ORDER_COLOUR, 1e-6), (64, ORDER_REFERENCE, 1e-12)):
        p = sc.params()
        p.solve_to_tolerance = 1
        p.residual_tolerance = tol
        p.max_iterations_to_tolerance = 4000
        o = OracleWorld(p, sc.gravity, precision=prec, order=order)
        o.load_scene(sc)
        o.step(1)
        cs = o.contacts()
        order_ = np.argsort(cs["collider2"])
        out.append(o.contacts_f64()[order_, 10])
    m = 4.0 / 3.0 * np.pi * 0.5 ** 3
    statics = (k - np.arange(k)) * m * 9.81 / 60.0
    np.testing.assert_allclose(out[0], out[1], rtol=1e-4)
    np.testing.assert_allclose(out[1], statics, rtol=1e-6)


def test_capsule_mass_properties_follow_the_reference_formula():
    # volumetric_capsule.rs:7-37 (with volumetric_cylinder.rs:7-60 and
    # volumetric_ball.rs): volume = cylinder + ball; unit inertia = the
    # cylinder's + the ball's + (h^2 / 2 + h r 3/8) on x and z, h = 2 half
    # height; inertia = unit inertia x mass. Checked in f64 against that
    # formula written out here, for a capsule turned about z by 30 degrees.
    r, hh, rho = 0.35, 0.9, 2.5
    vol = hh * r * r * math.pi * 2 + math.pi * r ** 3 * 4.0 / 3.0
    m = vol * rho
    off = (3 * r * r + 4 * hh * hh) / 12.0
    diag = 0.4 * r * r
    h = 2 * hh
    extra = h * h * 0.5 + h * r * 3.0 / 8.0
    unit = np.diag([off + diag + extra, r * r / 2 + diag, off + diag + extra])
    a = math.radians(30.0)
    R = np.array([[math.cos(a), -math.sin(a), 0], [math.sin(a), math.cos(a), 0], [0, 0, 1]])
    want = R @ (unit * m) @ R.T
    b = scenes.body_descs(1)
    c = scenes.collider_descs(1, 0, abi.SHAPE_CAPSULE, (r, hh, 0), density=rho)
    c["position_wrt_body"][0, 3:] = (0.0, 0.0, math.sin(a / 2), math.cos(a / 2))
    o = OracleWorld(scenes.Scene("capsule", b, c).params(), (0.0, 0.0, 0.0), precision=64)
    o.load_scene(scenes.Scene("capsule", b, c, gravity=(0.0, 0.0, 0.0)))
    o.step(1)
    inertia, com = o.mass_properties()
    assert abs(inertia[0, 0] - m) <= 1e-6 * m
    got = np.array([[inertia[0, 1], inertia[0, 2], inertia[0, 3]], [inertia[0, 2], inertia[0, 4], inertia[0, 5]],
                    [inertia[0, 3], inertia[0, 5], inertia[0, 6]]])
    np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(com[0], 0.0, atol=1e-7)


def test_capsule_comes_to_rest_lying_on_the_ground():
    # A capsule dropped at a tilt onto the ground tumbles and comes to rest
    # on its side: its axis horizontal, its centre one radius above the
    # ground (f32 oracle, the GPU's colour order).
    r, hh = 0.3, 0.7
    sc = scenes.single_body(shape=abi.SHAPE_CAPSULE, params=(r, hh, 0), position=(0, 2.0, 0),
                            rotation=(0.0, 0.0, math.sin(0.3), math.cos(0.3)))
    o = OracleWorld(sc.params(), sc.gravity, precision=32, order=ORDER_COLOUR)
    o.load_scene(sc)
    o.step(400)
    pos = o.bodies()["position"][1]
    assert abs(pos[1] - r) < 0.02, pos
    q = pos[3:]
    # The capsule's axis (its local y) in world coordinates is horizontal.
    yaxis = np.array([2 * (q[0] * q[1] - q[2] * q[3]), 1 - 2 * (q[0] ** 2 + q[2] ** 2), 2 * (q[1] * q[2] + q[0] * q[3])])
    assert abs(yaxis[1]) < 0.05, yaxis

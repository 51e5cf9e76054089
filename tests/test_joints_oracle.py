"""Joint constraints in the CPU oracle (no GPU).

BallConstraint and FixedConstraint (src/joint/ball_constraint.rs,
fixed_constraint.rs) as the reference assembles them: bilateral rows of
ImpulseLimits::Independent (helper.rs:167-296, 422-551) solved with the
friction rows by SORProx (sor_prox.rs:159-179), position rows solved by
NonlinearSORProx::solve_generic (nonlinear_sor_prox.rs:78-117), impulses
cached by the joint and checked against the break force. The checks are
analytic: a pendulum's period, a hanging chain's statics, a fixed pair
keeping its relative pose, orders converging to one solution, breaking,
removal and islands.
"""
import math

import numpy as np
import pytest

from nphysics_gb300 import abi, scenes
from oracle.oracle_py import ORDER_COLOUR, ORDER_REFERENCE, OracleWorld


def _rot(q, v):
    u, w = np.asarray(q[:3], np.float64), float(q[3])
    t = 2.0 * np.cross(u, v)
    return np.asarray(v, np.float64) + w * t + np.cross(u, t)


def _qmul(a, b):
    return scenes._qmul(np.asarray(a, np.float64), np.asarray(b, np.float64))


def _joint_errors(sc, pos):
    """Anchor separation of every joint, and the frames' relative rotation
    angle of every fixed joint."""
    lin, ang = [], []
    for j in sc.joints:
        i1, i2 = int(j["body1"]["index"]), int(j["body2"]["index"])
        p1 = pos[i1] if sc.bodies["kind"][i1] != abi.KIND_GROUND else np.array([0, 0, 0, 0, 0, 0, 1.0])
        a1 = p1[:3] + _rot(p1[3:7], j["anchor1"])
        a2 = pos[i2, :3] + _rot(pos[i2, 3:7], j["anchor2"])
        lin.append(np.linalg.norm(a1 - a2))
        if j["kind"] == abi.JOINT_FIXED:
            r1 = _qmul(p1[3:7], j["frame1"])
            r2 = _qmul(pos[i2, 3:7], j["frame2"])
            d = _qmul(r2, scenes._qconj(r1))
            ang.append(2 * math.acos(min(1.0, abs(d[3]))))
    return np.array(lin), np.array(ang)


@pytest.mark.parametrize("precision", [32, 64])
def test_pendulum_period_and_rod_length(precision):
    # A ball on a 2 m rod released at 0.1 rad: T = 2 pi sqrt(L / g) (1 + theta^2 / 16)
    # to second order in the amplitude; the rod stretches by at most 4 mm at
    # the bottom of the swing (measured 2.7 mm in f32, 2.0 mm in f64: the
    # allowed linear error of 1 mm plus what three position iterations at
    # erp 0.2 leave of each step's drift).
    sc = scenes.pendulum(length=2.0, angle=0.1)
    w = OracleWorld(sc.params(), sc.gravity, precision=precision)
    w.load_scene(sc)
    xs, rod = [], []
    for _ in range(600):
        w.step(1)
        p = w.bodies()["position"][1, :3]
        xs.append(p[0])
        rod.append(np.linalg.norm(p - np.array([0.0, 10.0, 0.0])))
    xs = np.array(xs)
    crossings = [i for i in range(1, len(xs)) if xs[i - 1] > 0 >= xs[i]]
    period = np.diff(crossings).mean() / 60.0
    expected = 2 * math.pi * math.sqrt(2.0 / 9.81) * (1 + 0.1 ** 2 / 16)
    assert abs(period - expected) < 0.004 * expected
    assert max(abs(r - 2.0) for r in rod) < 4e-3


def test_hanging_chain_impulses_carry_the_weight_below():
    # Three balls hanging at rest, solved to a tight residual: joint i carries
    # the weight of the balls below it, (3 - i) m g dt along y.
    sc = scenes.pendulum(length=1.0, angle=0.0, chain=3)
    p = sc.params()
    p.solve_to_tolerance = 1
    p.residual_tolerance = 1e-9
    p.max_iterations_to_tolerance = 2000
    w = OracleWorld(p, sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(30)
    imp, broken, active = w.joints(sc.joint_handles)
    m = 4.0 / 3.0 * math.pi * float(np.float32(0.1)) ** 3 * 100.0
    dt = float(np.float32(1.0 / 60.0))
    g = float(np.float32(9.81))
    for i in range(3):
        assert abs(abs(imp[i, 1]) - (3 - i) * m * g * dt) < 1e-6 * (3 - i) * m * g * dt
        assert abs(imp[i, 0]) < 1e-9 and abs(imp[i, 2]) < 1e-9
    assert not broken.any() and active.all()


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("order", [ORDER_REFERENCE, ORDER_COLOUR])
def test_joints_hold_through_swings_and_impacts(precision, order):
    # Chains swinging onto the ground and fixed pairs tumbling onto it, with
    # the default 8 velocity / 3 position iterations: every anchor pair stays
    # within 6 cm and every fixed frame within 0.15 rad over 300 steps
    # (measured at most 4.0 cm and 0.092 rad: an 8-link chain is a long
    # Gauss-Seidel chain, and links pressed on the ground or against each
    # other at their joints contend with the joints).
    sc = scenes.jointed()
    w = OracleWorld(sc.params(), sc.gravity, precision=precision, order=order)
    w.load_scene(sc)
    for _ in range(6):
        w.step(50)
        lin, ang = _joint_errors(sc, w.bodies()["position"])
        assert lin.max() < 0.06
        assert ang.max() < 0.15
    assert w.counters()["num_contacts"] > 20


def _lifted(**kw):
    sc = scenes.jointed(**kw)
    sc.bodies["position"][1:, 1] += 60.0
    sc.joints["anchor1"][:, 1] += np.where(sc.joints["body1"]["index"] == 0, 60.0, 0.0)
    return sc


def _max_error(sc, velocity_iterations, position_iterations, steps=120):
    p = sc.params()
    p.max_velocity_iterations = velocity_iterations
    p.max_position_iterations = position_iterations
    w = OracleWorld(p, sc.gravity, precision=64)
    w.load_scene(sc)
    lin_max, ang_max = 0.0, 0.0
    for _ in range(steps):
        w.step(1)
        lin, ang = _joint_errors(sc, w.bodies()["position"])
        lin_max = max(lin_max, lin.max())
        ang_max = max(ang_max, ang.max() if len(ang) else 0.0)
    return lin_max, ang_max


def test_joint_errors_fall_with_iterations_away_from_contacts():
    # Swinging chains high above the ground: the stretch falls as the
    # iterations grow (measured 3.3 cm, 0.76 cm, 0.41 cm).
    sc = _lifted(chains=4, links=8, clusters=0, balls=0)
    e = [_max_error(sc, v, q)[0] for v, q in ((8, 3), (50, 20), (200, 50))]
    assert e[0] > e[1] > e[2]
    assert e[2] < 0.006
    # Tumbling fixed pairs in free fall stay at the allowed errors: the
    # position rows skip errors below allowed_linear_error (1 mm) and
    # allowed_angular_error (1 mrad).
    lin, ang = _max_error(_lifted(chains=0, clusters=6, balls=0), 8, 3)
    assert lin < 1.1e-3 and ang < 1.0e-3


def test_orders_converge_to_the_same_velocities_with_joints():
    # The reference's order (joints first, sor_prox.rs:159-179), the colour
    # order and the per-manifold order are Gauss-Seidel orders of the same
    # rows: solved to a tight residual they agree.
    sc = scenes.jointed(chains=2, links=5, clusters=3, balls=4)
    out = []
    for order, sweep in ((ORDER_REFERENCE, abi.SWEEP_SEPARATE), (ORDER_COLOUR, abi.SWEEP_SEPARATE),
                         (ORDER_COLOUR, abi.SWEEP_MANIFOLD)):
        p = sc.params()
        p.max_position_iterations = 0
        p.solve_to_tolerance = 1
        p.residual_tolerance = 1e-11
        p.max_iterations_to_tolerance = 20000
        p.sweep_order = sweep
        w = OracleWorld(p, sc.gravity, precision=64, order=order)
        w.load_scene(sc)
        w.step(1)
        assert w.counters()["residual"] <= 1e-11
        out.append(w.bodies()["velocity"])
    np.testing.assert_allclose(out[0], out[1], atol=1e-7)
    np.testing.assert_allclose(out[0], out[2], atol=1e-7)


def test_a_joint_breaks_above_its_break_force_and_the_body_falls_free():
    # The ball weighs m g = 4.1 N: a 1 N break force fails at the first step
    # (|impulse|^2 / dt^2 > 1), after which the ball falls freely.
    sc = scenes.pendulum(length=2.0, angle=0.0)
    sc.joints["break_force"] = 1.0
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(1)
    _, broken, _ = w.joints(sc.joint_handles)
    assert broken[0]
    v0 = w.bodies()["velocity"][1, 1]
    w.step(10)
    _, _, active = w.joints(sc.joint_handles)
    assert not active[0]
    v1 = w.bodies()["velocity"][1, 1]
    assert abs((v1 - v0) - (-9.81 * 10 / 60.0)) < 1e-4


def test_removing_a_joint_or_its_body():
    sc = scenes.pendulum(length=1.0, angle=0.0, chain=2)
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(20)
    y = w.bodies()["position"][2, 1]
    # Removing the lower joint: the lower ball falls, the upper one stays.
    w.remove_joints(sc.joint_handles[1:2])
    w.step(20)
    b = w.bodies()["position"]
    assert b[2, 1] < y - 0.5
    assert abs(np.linalg.norm(b[1, :3] - np.array([0.0, 10.0, 0.0])) - 1.0) < 2e-3
    with pytest.raises(RuntimeError):
        w.joints(sc.joint_handles[1:2])
    # Removing the upper ball removes its joint too.
    w.remove_bodies(sc.body_handles[1:2])
    with pytest.raises(RuntimeError):
        w.joints(sc.joint_handles[0:1])


def test_a_jointed_chain_sleeps_and_wakes_as_one_island():
    # Joints join islands (activation_manager.rs:154-159): a resting chain
    # sleeps together, and a force on its lowest ball wakes every ball.
    sc = scenes.pendulum(length=1.0, angle=0.0, chain=3)
    sc.bodies["flags"][1:] = abi.BODY_GRAVITY | abi.BODY_CAN_SLEEP
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(400)
    assert not w.bodies()["active"][1:].any()
    w.apply_forces(sc.body_handles[3:4], np.array([[5.0, 0, 0, 0, 0, 0]], np.float32), wake=True)
    w.step(1)
    assert w.bodies()["active"][1:].all()


def _angle_about_z(q):
    return 2.0 * math.atan2(q[2], q[3])


@pytest.mark.parametrize("precision", [32, 64])
def test_revolute_hinge_is_a_physical_pendulum(precision):
    # A 1 x 0.2 x 0.2 box hinged at one end about z, released 0.15 rad from
    # the vertical, swings as a physical pendulum about the pivot:
    # T = 2 pi sqrt(I_p / (m g d)) (1 + theta^2 / 16), with
    # I_p = m (a^2 + b^2) / 3 + m a^2 and d = a (half length a, half height b);
    # measured 0.1 % short, the amplitude kept to 2e-4 rad over six swings. It
    # stays in the x-y plane.
    a, b = 0.5, 0.1
    sc = scenes.hinge(kind=abi.JOINT_REVOLUTE, half=(a, b, 0.1), angle=math.pi / 2 - 0.15)
    w = OracleWorld(sc.params(), sc.gravity, precision=precision)
    w.load_scene(sc)
    th, out_of_plane = [], 0.0
    for _ in range(600):
        w.step(1)
        p = w.bodies()["position"][1]
        th.append(_angle_about_z(p[3:7]))
        out_of_plane = max(out_of_plane, abs(p[2]), abs(p[3]), abs(p[4]))
    th = np.array(th) + math.pi / 2          # swing angle from the vertical
    crossings = [i for i in range(1, len(th)) if th[i - 1] > 0 >= th[i]]
    period = np.diff(crossings).mean() / 60.0
    ip = (a * a + b * b) / 3 + a * a
    expected = 2 * math.pi * math.sqrt(ip / (9.81 * a)) * (1 + 0.15 ** 2 / 16)
    assert abs(period - expected) < 0.01 * expected
    assert out_of_plane < 1e-3


def test_cartesian_joint_keeps_the_orientation_and_frees_the_translation():
    # CartesianConstraint locks the relative rotation only: a spinning box
    # held by one to the ground stops turning and falls freely.
    sc = scenes.hinge(kind=abi.JOINT_CARTESIAN, angle=0.0, spin=(0.0, 0.0, 0.0))
    sc.bodies["velocity"][1] = (1.0, 0.0, 0.0, 0.0, 3.0, 2.0)
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(30)
    b = w.bodies()
    q = b["position"][1, 3:7]
    assert 2 * math.acos(min(1.0, abs(q[3]))) < 0.01
    assert np.abs(b["velocity"][1, 3:]).max() < 1e-3
    assert abs(b["velocity"][1, 1] - (-9.81 * 30 / 60.0)) < 0.01


def test_planar_joint_keeps_the_body_in_its_plane():
    # PlanarConstraint: anchor2 stays in the plane through anchor1 normal to
    # axis1 (y here), and the body turns only about the axis.
    sc = scenes.hinge(kind=abi.JOINT_PLANAR, angle=0.0)
    sc.joints["axis1"][0] = (0.0, 1.0, 0.0)
    sc.joints["axis2"][0] = (0.0, 1.0, 0.0)
    sc.bodies["velocity"][1] = (1.0, -2.0, 0.5, 1.0, 2.0, -1.0)
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    for _ in range(4):
        w.step(30)
        p = w.bodies()["position"][1]
        a2 = p[:3] + _rot(p[3:7], sc.joints["anchor2"][0])
        assert abs(a2[1] - 10.0) < 2e-3
        y_axis = _rot(p[3:7], np.array([0.0, 1.0, 0.0]))
        assert math.acos(min(1.0, y_axis[1])) < 0.01
    v = w.bodies()["velocity"][1]
    assert abs(v[0]) > 0.5 and abs(v[4]) > 0.5          # it slides and turns about y


def test_rectangular_joint_translates_in_its_plane_without_turning():
    sc = scenes.hinge(kind=abi.JOINT_RECTANGULAR, angle=0.0)
    sc.joints["axis1"][0] = (0.0, 0.0, 1.0)             # the plane normal: z
    sc.bodies["velocity"][1] = (0.5, 1.0, 2.0, 1.0, 1.0, 1.0)
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(60)
    p = w.bodies()["position"][1]
    a2 = p[:3] + _rot(p[3:7], sc.joints["anchor2"][0])
    assert abs(a2[2]) < 2e-3
    assert 2 * math.acos(min(1.0, abs(p[6]))) < 0.01
    assert p[1] < 9.0                                    # it falls within its plane


def test_universal_joint_keeps_the_angle_between_its_axes():
    # Two bodies joined at a point, body 1's x axis and body 2's y axis kept
    # at 90 degrees while the pair tumbles.
    sc = scenes.joint_zoo()
    k = int(np.nonzero(sc.joints["kind"] == abi.JOINT_UNIVERSAL)[0][0])
    j = sc.joints[k]
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    for _ in range(8):
        w.step(30)
        pos = w.bodies()["position"]
        i1, i2 = int(j["body1"]["index"]), int(j["body2"]["index"])
        a1 = _rot(pos[i1, 3:7], j["axis1"])
        a2 = _rot(pos[i2, 3:7], j["axis2"])
        ang = math.acos(max(-1.0, min(1.0, float(np.dot(a1, a2)))))
        assert abs(ang - math.pi / 2) < 0.02
        p1 = pos[i1, :3] + _rot(pos[i1, 3:7], j["anchor1"])
        p2 = pos[i2, :3] + _rot(pos[i2, 3:7], j["anchor2"])
        assert np.linalg.norm(p1 - p2) < 0.01


def test_every_joint_kind_converges_to_one_solution_in_every_order():
    sc = scenes.joint_zoo()
    out = []
    for order, sweep in ((ORDER_REFERENCE, abi.SWEEP_SEPARATE), (ORDER_COLOUR, abi.SWEEP_SEPARATE),
                         (ORDER_COLOUR, abi.SWEEP_MANIFOLD)):
        p = sc.params()
        p.max_position_iterations = 0
        p.solve_to_tolerance = 1
        p.residual_tolerance = 1e-11
        p.max_iterations_to_tolerance = 20000
        p.sweep_order = sweep
        w = OracleWorld(p, sc.gravity, precision=64, order=order)
        w.load_scene(sc)
        w.step(1)
        assert w.counters()["residual"] <= 1e-11
        out.append(w.bodies()["velocity"])
    np.testing.assert_allclose(out[0], out[1], atol=1e-7)
    np.testing.assert_allclose(out[0], out[2], atol=1e-7)


def _slider(kind, axis, velocity, **limits):
    sc = scenes.hinge(kind=kind, angle=0.0)
    sc.joints["axis1"][0] = axis
    sc.joints["axis2"][0] = axis
    sc.bodies["velocity"][1] = velocity
    flags = 0
    if "min_offset" in limits:
        flags |= abi.JOINT_MIN_OFFSET
        sc.joints["min_offset"][0] = limits["min_offset"]
    if "max_offset" in limits:
        flags |= abi.JOINT_MAX_OFFSET
        sc.joints["max_offset"][0] = limits["max_offset"]
    sc.joints["limit_flags"][0] = flags
    return sc


def test_prismatic_slider_rests_on_its_offset_limit():
    # A vertical slider falls along its axis onto its lower limit (offset
    # -1): it rests 1 m below the pivot, within the allowed error, and the
    # limit carries its weight, m g dt, once solved to a tight residual.
    sc = _slider(abi.JOINT_PRISMATIC, (0.0, 1.0, 0.0), (0, 0, 0, 0, 0, 0), min_offset=-1.0, max_offset=0.5)
    p = sc.params()
    p.solve_to_tolerance = 1
    p.residual_tolerance = 1e-10
    p.max_iterations_to_tolerance = 2000
    w = OracleWorld(p, sc.gravity, precision=64)
    w.load_scene(sc)
    w.step(120)
    pos = w.bodies()["position"][1]
    anchor2 = pos[:3] + _rot(pos[3:7], sc.joints["anchor2"][0])
    assert abs(anchor2[1] - 9.0) < 2e-3
    assert abs(anchor2[0]) < 1e-6 and abs(anchor2[2]) < 1e-6
    imp = w.joints(sc.joint_handles)[0][0]
    m = 1.0 * 0.5 * 0.1 * 0.1 * 8 * float(np.float32(1.0))
    assert abs(imp[6] - m * 9.81 / 60.0) < 1e-4 * m * 9.81 / 60.0


def test_prismatic_slider_slides_to_its_upper_limit_without_falling():
    sc = _slider(abi.JOINT_PRISMATIC, (1.0, 0.0, 0.0), (2.0, 0, 0, 0, 0, 0), min_offset=-0.5, max_offset=0.5)
    w = OracleWorld(sc.params(), sc.gravity, precision=64)
    w.load_scene(sc)
    hit = False
    for _ in range(60):
        w.step(1)
        pos = w.bodies()["position"][1]
        a2 = pos[:3] + _rot(pos[3:7], sc.joints["anchor2"][0])
        assert abs(a2[1] - 10.0) < 3e-3 and abs(a2[2]) < 1e-6
        assert a2[0] < 0.5 + 0.05
        hit = hit or w.joints(sc.joint_handles)[0][0][6] > 0
    assert hit
    assert abs(a2[0] - 0.5) < 0.01


@pytest.mark.parametrize("kind", [abi.JOINT_CYLINDRICAL, abi.JOINT_PIN_SLOT])
def test_cylindrical_and_pin_slot_joints_slide_and_turn_about_their_axes(kind):
    # Both free the translation along axis1 (x) and one rotation: about x for
    # the cylindrical joint, about axis3 = axis2 (z) for the pin-slot, which
    # then swings as a pendulum on its sliding pin. A body started sliding
    # along x and spinning about every axis keeps its anchor on the x line
    # (measured within 2.4 mm and 7.4 mm at 8 / 3 iterations, 0 and 1.1 mm at
    # 50 / 20) and turns about its free axis only.
    def run(vi, pi):
        sc = _slider(kind, (1.0, 0.0, 0.0), (1.0, 0.0, 0.0, 2.0, 2.0, 2.0))
        if kind == abi.JOINT_PIN_SLOT:
            sc.joints["axis3"][0] = (0.0, 0.0, 1.0)
            sc.joints["axis2"][0] = (0.0, 0.0, 1.0)
        p = sc.params()
        p.max_velocity_iterations, p.max_position_iterations = vi, pi
        w = OracleWorld(p, sc.gravity, precision=64)
        w.load_scene(sc)
        off = 0.0
        for _ in range(30):
            w.step(1)
            pos = w.bodies()["position"][1]
            a2 = pos[:3] + _rot(pos[3:7], sc.joints["anchor2"][0])
            off = max(off, abs(a2[1] - 10.0), abs(a2[2]))
        return off, a2, w.bodies()["velocity"][1]

    off, a2, vel = run(8, 3)
    assert off < 0.01 and a2[0] > 0.3
    free, locked = (3, (4, 5)) if kind == abi.JOINT_CYLINDRICAL else (5, (3, 4))
    assert abs(vel[free]) > 1.0 and max(abs(vel[k]) for k in locked) < 5e-3
    off, _, _ = run(50, 20)
    assert off < 1.2e-3

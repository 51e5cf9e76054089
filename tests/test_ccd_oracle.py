"""Continuous collision detection in the oracle (CPU): the distance and
time-of-impact geometry against independent references, and the CCD
substeps of MechanicalWorld::solve_ccd (src/world/mechanical_world.rs:398-1052)
on known-answer scenes: fast projectiles through a thin wall, a tower struck
by fast balls, resting CCD bodies, substep counts and the penetration switch.
"""
import math

import numpy as np
import pytest
from scipy.optimize import minimize, minimize_scalar

from nphysics_gb300 import abi, scenes
from oracle.oracle_py import ORDER_COLOUR, ORDER_REFERENCE, OracleWorld


def two(shape1, p1, pos1, q1, shape2, p2, pos2, q2, vel1=(0, 0, 0, 0, 0, 0), vel2=(0, 0, 0, 0, 0, 0), prec=64):
    b = scenes.body_descs(2)
    b["flags"] = 0
    b["position"][0, :3], b["position"][0, 3:] = pos1, q1
    b["position"][1, :3], b["position"][1, 3:] = pos2, q2
    b["velocity"][0], b["velocity"][1] = vel1, vel2
    c = np.concatenate([scenes.collider_descs(1, 0, shape1, p1, density=1.0),
                        scenes.collider_descs(1, 1, shape2, p2, density=1.0)])
    sc = scenes.Scene("two", b, c, gravity=(0, 0, 0))
    o = OracleWorld(sc.params(), sc.gravity, precision=prec)
    o.load_scene(sc)
    return o


def qmat(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def box_point(p, c, R, h):
    loc = R.T @ (p - c)
    return np.linalg.norm(loc - np.clip(loc, -h, h))


def box_box(c1, R1, h1, c2, R2, h2):
    # The distance from box 2 is convex over box 1: Nelder-Mead from several starts.
    f = lambda u: box_point(c1 + R1 @ (np.tanh(u) * h1), c2, R2, h2)
    rng = np.random.default_rng(0)
    return min(minimize(f, rng.normal(size=3), method="Nelder-Mead",
                        options={"xatol": 1e-10, "fatol": 1e-12, "maxiter": 4000}).fun for _ in range(12))


@pytest.mark.parametrize("prec,tol", [(64, 1e-6), (32, 2e-5)])
def test_distance_of_cuboids_balls_and_capsules(prec, tol):
    # Gilbert-Johnson-Keerthi on the shapes' cores against a direct
    # minimisation: cuboid-cuboid, ball-cuboid and capsule-cuboid pairs at
    # random poses, each separated.
    rng = np.random.default_rng(1)
    for trial in range(24):
        q1, q2 = (scenes.uniform_quaternions(rng, 1)[0].astype(np.float64) for _ in range(2))
        h1, h2 = rng.uniform(0.2, 1.0, 3), rng.uniform(0.2, 1.0, 3)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        pos2 = d * rng.uniform(2.5, 4.0)
        kind = trial % 3
        if kind == 0:
            o = two(abi.SHAPE_CUBOID, h1, (0, 0, 0), q1, abi.SHAPE_CUBOID, h2, pos2, q2, prec=prec)
            ref = box_box(np.zeros(3), qmat(q1), h1, pos2, qmat(q2), h2)
        elif kind == 1:
            o = two(abi.SHAPE_BALL, (0.1, 0, 0), (0, 0, 0), (0, 0, 0, 1), abi.SHAPE_CUBOID, h2, pos2, q2, prec=prec)
            ref = box_point(np.zeros(3), pos2, qmat(q2), h2) - 0.1
        else:
            o = two(abi.SHAPE_CAPSULE, (0.1, 0.5, 0), (0, 0, 0), q1, abi.SHAPE_CUBOID, h2, pos2, q2, prec=prec)
            axis = qmat(q1) @ np.array([0.0, 1.0, 0.0])
            ref = minimize_scalar(lambda s: box_point(axis * s, pos2, qmat(q2), h2), bounds=(-0.5, 0.5),
                                  method="bounded", options={"xatol": 1e-12}).fun - 0.1
        dist, n = o.collider_distance(0, 1)
        assert abs(dist - ref) < tol, (trial, dist, ref)
        assert abs(np.linalg.norm(n) - 1.0) < 1e-5


def test_distance_of_overlapping_shapes_is_negative():
    o = two(abi.SHAPE_BALL, (0.5, 0, 0), (0, 0, 0), (0, 0, 0, 1), abi.SHAPE_BALL, (0.5, 0, 0), (0.8, 0, 0), (0, 0, 0, 1))
    assert o.collider_distance(0, 1)[0] == pytest.approx(-0.2, abs=1e-6)
    o = two(abi.SHAPE_CUBOID, (0.5, 0.5, 0.5), (0, 0, 0), (0, 0, 0, 1), abi.SHAPE_CUBOID, (0.5, 0.5, 0.5), (0.9, 0, 0),
            (0, 0, 0, 1))
    assert o.collider_distance(0, 1)[0] <= 0.0


@pytest.mark.parametrize("prec", [32, 64])
def test_time_of_impact_of_a_translating_ball(prec):
    # A ball 1 m from a cuboid's face closing at 50 m/s: one advancement to
    # half the target distance, so the TOI is (d0 - target / 2) / v.
    o = two(abi.SHAPE_BALL, (0.1, 0, 0), (-1.1, 0, 0), (0, 0, 0, 1), abi.SHAPE_CUBOID, (0.05, 1, 1), (0, 0, 0),
            (0, 0, 0, 1), vel1=(50, 0, 0, 0, 0, 0), prec=prec)
    status, toi = o.pair_toi(0, 1, 1.0)
    assert status == 0
    assert toi == pytest.approx((0.95 - 0.0005) / 50.0, rel=1e-5)
    # Out of reach within the horizon, moving apart, already overlapping.
    assert o.pair_toi(0, 1, 0.01)[0] == -1
    o = two(abi.SHAPE_BALL, (0.1, 0, 0), (-1.1, 0, 0), (0, 0, 0, 1), abi.SHAPE_CUBOID, (0.05, 1, 1), (0, 0, 0),
            (0, 0, 0, 1), vel1=(-50, 0, 0, 0, 0, 0), prec=prec)
    assert o.pair_toi(0, 1, 1.0)[0] == -1
    o = two(abi.SHAPE_BALL, (0.1, 0, 0), (-0.1, 0, 0), (0, 0, 0, 1), abi.SHAPE_CUBOID, (0.05, 1, 1), (0, 0, 0),
            (0, 0, 0, 1), vel1=(50, 0, 0, 0, 0, 0), prec=prec)
    assert o.pair_toi(0, 1, 1.0) == (1, 0.0)


def test_time_of_impact_of_spinning_cuboids_is_conservative():
    # A spinning cuboid thrown at another: at the TOI the shapes are within
    # the target distance, and never touched before it.
    rng = np.random.default_rng(4)
    for trial in range(12):
        q1, q2 = (scenes.uniform_quaternions(rng, 1)[0].astype(np.float64) for _ in range(2))
        w = rng.normal(size=3) * 20.0
        v = np.array([30.0, rng.normal(), rng.normal()])
        args = (abi.SHAPE_CUBOID, (0.3, 0.2, 0.1), (-2.0, 0, 0), q1, abi.SHAPE_CUBOID, (0.2, 0.5, 0.5), (0, 0, 0), q2)
        o = two(*args, vel1=tuple(v) + tuple(w))
        status, toi = o.pair_toi(0, 1, 0.5)
        assert status == 0, trial
        # The pose at time s: a fresh world displaced by the motion.
        def dist_at(s):
            from oracle.oracle_py import OracleWorld as _W  # noqa: F401
            ob = two(*args, vel1=tuple(v) + tuple(w))
            p = ob.bodies()["position"][0]
            ang = np.linalg.norm(w * s)
            axis = w / np.linalg.norm(w)
            dq = np.concatenate([axis * math.sin(ang / 2), [math.cos(ang / 2)]])
            x, y, z, ww = dq
            a1, b1, c1, d1 = p[3:]
            q = np.array([ww * a1 + x * d1 + y * c1 - z * b1, ww * b1 - x * c1 + y * d1 + z * a1,
                          ww * c1 + x * b1 - y * a1 + z * d1, ww * d1 - x * a1 - y * b1 - z * c1])
            ob.set_body_state(0, pos=np.concatenate([p[:3] + v * s, q])[None].astype(np.float32))
            return ob.collider_distance(0, 1)[0]
        assert 0.0 < dist_at(toi) <= 0.0011, trial
        assert min(dist_at(s) for s in np.linspace(0.0, toi, 40)) > 0.0, trial


def run(scene, steps, order=ORDER_COLOUR, prec=32, **kw):
    p = scene.params()
    for k, v in kw.items():
        setattr(p, k, v)
    o = OracleWorld(p, scene.gravity, precision=prec, order=order)
    o.load_scene(scene)
    sub = imp = 0
    for _ in range(steps):
        o.step(1)
        c = o.counters()
        sub += c["ccd_substeps"]
        imp += c["ccd_impacts"]
    return o, sub, imp


@pytest.mark.parametrize("shape,spin", [(abi.SHAPE_BALL, 0.0), (abi.SHAPE_CUBOID, 0.0), (abi.SHAPE_CUBOID, 40.0)])
def test_fast_projectiles_do_not_tunnel_through_a_thin_wall(shape, spin):
    # 2 m a step against a wall 10 cm thick: without CCD every projectile is
    # past the wall after one step; with CCD each stops on the near side in
    # one substep (restitution 0).
    kw = dict(shape=shape, spin=spin, n=4)
    o, sub, imp = run(scenes.ccd_wall(ccd=False, **kw), 3)
    assert (o.bodies()["position"][1:, 0] > 0.05).all() and sub == 0
    o, sub, imp = run(scenes.ccd_wall(ccd=True, **kw), 3)
    x = o.bodies()["position"][1:, 0]
    assert (x < -0.05).all(), x
    assert sub >= 1 and imp >= 4
    if spin == 0.0:
        assert (x > -0.2).all() and np.abs(o.bodies()["velocity"][1:, 0]).max() < 0.05


@pytest.mark.parametrize("prec", [32, 64])
def test_ccd_balls_stay_outside_a_struck_tower(prec):
    # Fast CCD balls into a tower of boxes: never inside a box at the end of
    # a step (without CCD some pass through), and an impact for each ball.
    def inside(o):
        b = o.bodies()
        boxes, balls = b["position"][1:5], b["position"][5:]
        worst = 1.0
        for bp in balls:
            for q in boxes:
                loc = qmat(q[3:].astype(np.float64)).T @ (bp[:3] - q[:3])
                worst = min(worst, float(np.max(np.abs(loc)) - 0.5))
        return worst
    o, sub, imp = run(scenes.ccd_stack(), 30, prec=prec)
    assert sub >= 1 and imp >= 3
    o2, _, _ = run(scenes.ccd_stack(), 1, prec=prec)
    for _ in range(40):
        o2.step(1)
        assert inside(o2) > -0.21   # a ball's centre never deeper than its radius (0.2) in a box


def test_resting_ccd_body_and_disabled_ccd():
    # A CCD cube resting on the ground stays at rest; max_ccd_substeps = 0
    # turns CCD off (the fast ball then passes the wall).
    sc = scenes.single_body(position=(0, 0.5, 0))
    sc.colliders["ccd_enabled"][1] = 1
    o, sub, imp = run(sc, 120)
    b = o.bodies()
    assert abs(b["position"][1, 1] - 0.5) < 0.03 and np.abs(b["velocity"][1]).max() < 1e-2
    o, sub, _ = run(scenes.ccd_wall(), 2, max_ccd_substeps=0)
    assert sub == 0 and o.bodies()["position"][1, 0] > 0.05


def test_more_substeps_and_the_reference_order():
    # max_ccd_substeps = 4 splits the step; the reference and colour orders
    # both stop the balls (their main solves differ, the substeps do not).
    for order in (ORDER_REFERENCE, ORDER_COLOUR):
        o, sub, imp = run(scenes.ccd_wall(n=6), 3, order=order, max_ccd_substeps=4)
        assert sub >= 1 and imp >= 6
        assert (o.bodies()["position"][1:, 0] < -0.05).all()


def test_penetration_switch():
    # A CCD ball already overlapping the wall at the step's start: no impact
    # unless ccd_on_penetration_enabled, which resolves it at time zero.
    sc = scenes.ccd_wall(n=1)
    sc.bodies["position"][1, 0] = -0.1
    o, sub, _ = run(sc, 1)
    assert sub == 0
    o, sub, imp = run(sc, 1, ccd_on_penetration_enabled=1)
    assert sub == 1 and imp == 1


def test_f32_follows_f64():
    # The wall scene in both precisions: the same impacts and stops within
    # a millimetre.
    a, sa, ia = run(scenes.ccd_wall(n=4, gravity=(0, -9.81, 0)), 20, prec=32)
    b, sb, ib = run(scenes.ccd_wall(n=4, gravity=(0, -9.81, 0)), 20, prec=64)
    assert (sa, ia) == (sb, ib)
    np.testing.assert_allclose(a.bodies()["position"][:, :3], b.bodies()["position"][:, :3], atol=1e-3)


@pytest.mark.parametrize("prec", [32, 64])
def test_distance_of_parallel_features(prec):
    # Faces and axes parallel to a face: the configurations in which GJK's
    # simplex turns flat (resting boxes, a capsule lying against a wall).
    rng = np.random.default_rng(9)
    for trial in range(20):
        q = scenes.uniform_quaternions(rng, 1)[0].astype(np.float64)
        R = qmat(q)
        gap = rng.uniform(0.001, 0.05)
        h = np.array([0.5, 0.3, 0.2])
        # A cube resting on the first box's +x face, both rotated by q, shifted sideways.
        side = rng.uniform(-0.2, 0.2, 2)
        pos2 = R @ np.array([0.5 + 0.25 + gap, side[0], side[1]])
        o = two(abi.SHAPE_CUBOID, h, (0, 0, 0), q, abi.SHAPE_CUBOID, (0.25, 0.25, 0.25), pos2, q, prec=prec)
        assert o.collider_distance(0, 1)[0] == pytest.approx(gap, abs=2e-5 if prec == 32 else 1e-6), trial
        # A capsule (axis along the box's y) lying against the same face.
        pos3 = R @ np.array([0.5 + 0.1 + gap, side[0] * 0.5, side[1]])
        o = two(abi.SHAPE_CUBOID, h, (0, 0, 0), q, abi.SHAPE_CAPSULE, (0.1, 0.2, 0.0), pos3, q, prec=prec)
        assert o.collider_distance(0, 1)[0] == pytest.approx(gap, abs=2e-5 if prec == 32 else 1e-6), trial

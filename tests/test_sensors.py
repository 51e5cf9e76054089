"""Sensors and proximity events: a collider built with ColliderDesc::sensor
(src/object/collider.rs:542-543) is a proximity query. Its pairs make no
contacts and take no part in the solver or in CCD; their ncollide3d Proximity
(Intersecting, WithinMargin, Disjoint) is tracked per pass, and each change is
a ProximityEvent (GeometricalWorld::proximity_events,
src/world/geometrical_world.rs:378-381). The oracle's sensors are checked on
the CPU; the GPU against the oracle through the C ABI is marked gpu.
"""
import numpy as np
import pytest

from nphysics_gb300 import abi, scenes
from oracle.oracle_py import ORDER_COLOUR, OracleWorld

INT, WITHIN, DISJ = abi.PROXIMITY_INTERSECTING, abi.PROXIMITY_WITHIN_MARGIN, abi.PROXIMITY_DISJOINT


def oracle(scene, params=None):
    o = OracleWorld(params if params is not None else scene.params(), scene.gravity, precision=32,
                    order=ORDER_COLOUR)
    o.load_scene(scene)
    return o


def run_events(w, steps):
    out = []
    for _ in range(steps):
        w.step(1)
        out.append(w.proximity_events())
    return out


def test_sensors_do_not_change_the_motion():
    # No contacts and no mass: the bodies move as in the same scene without
    # the two sensor colliders, bit for bit.
    a, b = oracle(scenes.sensor_gates()), oracle(scenes.sensor_gates(sensors=False))
    for _ in range(12):
        a.step(10)
        b.step(10)
        np.testing.assert_array_equal(a.bodies()["position"], b.bodies()["position"])
        np.testing.assert_array_equal(a.bodies()["velocity"], b.bodies()["velocity"])


def test_zone_sees_every_ball_enter_and_leave():
    sc = scenes.sensor_gates()
    o = oracle(sc)
    o.enable_contact_events()
    ev = run_events(o, 150)
    zone, balls = 1, range(2, 2 + 6)
    state = {}
    for e in ev:
        for c1, c2, prev, new in e:
            assert prev != new
            assert state.get((c1, c2), DISJ) == prev   # each event starts where the last one ended
            state[(c1, c2)] = new
    for k in balls:
        seq = [(p, n) for e in ev for (c1, c2, p, n) in e if (c1, c2) == (zone, k)]
        assert seq and seq[0][0] == DISJ and INT in [n for _, n in seq], k
        assert seq[-1][1] == DISJ, k   # every ball fell through the zone to the ground
    # Contact events never involve a sensor.
    o.step(1)
    for c1, c2, _ in o.contact_events():
        assert zone not in (c1, c2) and 8 not in (c1, c2)


def test_moving_trigger_stays_on_the_ground():
    # The sensor ball around ball 0 (collider 8) reaches the ground and stays
    # Intersecting it while the ball rests there.
    o = oracle(scenes.sensor_gates())
    o.enable_contact_events()
    ev = run_events(o, 150)
    seq = [(p, n) for e in ev for (c1, c2, p, n) in e if (c1, c2) == (0, 8)]
    assert seq and seq[-1][1] == INT


def test_within_margin_between_apart_and_touching():
    # A ball lowered slowly onto a sensor slab passes through WithinMargin:
    # the pair's query limits are the ball's margin + linear prediction and
    # the sensor's linear prediction.
    g = scenes.ground_descs(1)
    gc = scenes.collider_descs(1, 0, abi.SHAPE_CUBOID, (2.0, 0.5, 2.0))
    gc["position_wrt_body"][0, 1] = -0.5
    gc["is_sensor"] = 1
    b = scenes.body_descs(1)
    b["position"][0, 1] = 0.3
    b["velocity"][0, 1] = -0.05
    c = scenes.collider_descs(1, 0, abi.SHAPE_BALL, (0.25, 0.0, 0.0), density=1.0)
    bodies, colliders = scenes._concat([g, b], [gc, c])
    sc = scenes.Scene("slow ball on a sensor slab", bodies, colliders, gravity=(0.0, 0.0, 0.0))
    o = oracle(sc)
    o.enable_contact_events()
    ev = [e for e in run_events(o, 120) if len(e)]
    seq = [(int(p), int(n)) for e in ev for (_, _, p, n) in e]
    assert seq[:2] == [(DISJ, WITHIN), (WITHIN, INT)], seq


def test_ccd_ignores_sensor_pairs():
    # A fast CCD ball crosses a thin sensor wall: no impact, no substep; it
    # moves as through empty space.
    sc = scenes.ccd_wall(n=2, ccd=True)
    sc.colliders["is_sensor"][0] = 1
    o = oracle(sc)
    o.step(3)
    assert o.counters()["ccd_substeps"] == 0
    x = o.bodies()["position"][1:, 0]
    assert (x > 0.5).all()


@pytest.mark.gpu
def test_gpu_sensors_match_oracle():
    from nphysics_gb300.world import GpuWorld
    sc = scenes.sensor_gates()
    p = sc.params()
    g, o = GpuWorld.for_scene(sc, p), oracle(sc, p)
    g.enable_contact_events()
    o.enable_contact_events()
    n_events = 0
    for _ in range(150):
        g.step(1)
        o.step(1)
        np.testing.assert_array_equal(g.bodies()["position"], o.bodies()["position"])
        np.testing.assert_array_equal(g.proximity_events(), o.proximity_events())
        np.testing.assert_array_equal(g.contact_events(), o.contact_events())
        n_events += len(g.proximity_events())
    assert n_events >= 12


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [0, 1])
def test_gpu_sensor_removal_and_graphs(graph):
    # Removing the zone gives no events for its pairs, as in the reference
    # (removal events are dropped before the step's first pass).
    from nphysics_gb300.world import GpuWorld
    sc = scenes.sensor_gates()
    p = sc.params()
    p.use_graph = graph
    g, o = GpuWorld.for_scene(sc, p), oracle(sc, p)
    g.enable_contact_events()
    o.enable_contact_events()
    for w in (g, o):
        w.step(45)
    h = sc.collider_handles[1:2]
    g.remove_colliders(h)
    o.remove_colliders(h)
    for _ in range(60):
        g.step(1)
        o.step(1)
        ge = g.proximity_events()
        np.testing.assert_array_equal(ge, o.proximity_events())
        assert not (ge[:, 0] == 1).any() if len(ge) else True
        np.testing.assert_array_equal(g.bodies()["position"], o.bodies()["position"])

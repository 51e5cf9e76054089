"""Geometric queries and contact events (GeometricalWorld::interferences_with_ray
/ _with_point / _with_aabb and contact_events, src/world/geometrical_world.rs:
327-376).

Known answers on the oracle (CPU): a ray's time of impact and normal on a ball
and on a rotated cuboid, a ray starting inside a shape, points inside and
outside, and the events of a ball that lands on the ground and is lifted off
again. On the GPU: the same known answers, and random batches of rays, points
and boxes over a cluster of balls and cuboids that equal the oracle's sets
(toi and normals within 1e-5), plus the events of a falling pile, step by
step, equal to the oracle's in the same Gauss-Seidel order.
"""
import math

import numpy as np
import pytest

from nphysics_gb300 import abi, scenes
from oracle.oracle_py import ORDER_COLOUR, OracleWorld


def _scene():
    # A static ball and a static rotated cuboid, nothing moving.
    b = scenes.body_descs(2)
    b["status"] = abi.BODY_STATIC
    b["position"][0, :3] = (0.0, 1.0, 0.0)
    a = math.radians(30.0)
    b["position"][1, :3] = (5.0, 1.0, 0.0)
    b["position"][1, 3:] = (0.0, math.sin(a / 2), 0.0, math.cos(a / 2))   # 30 degrees about y
    c = np.concatenate([scenes.collider_descs(1, 0, abi.SHAPE_BALL, (0.5, 0, 0), density=1.0),
                        scenes.collider_descs(1, 1, abi.SHAPE_CUBOID, (1.0, 0.5, 0.25), density=1.0)])
    return scenes.Scene("query known answers", b, c, gravity=(0.0, 0.0, 0.0))


def _world(backend, sc, events=False):
    if backend == "gpu":
        from nphysics_gb300.world import GpuWorld
        w = GpuWorld.for_scene(sc, sc.params())
    else:
        w = OracleWorld(sc.params(), sc.gravity, precision=32, order=ORDER_COLOUR)
        w.load_scene(sc)
    if events:
        w.enable_contact_events(1 << 16)
    return w


def _known_answers(backend):
    w = _world(backend, _scene())
    w.step(1)
    a = math.radians(30.0)
    rays = np.array([
        [-3.0, 1.0, 0.0, 2.0, 0.0, 0.0],            # along +x into the ball: hits at x = -0.5, toi 1.25
        [0.0, 1.0, 0.0, 0.0, 1.0, 0.0],             # from the ball's centre: inside, toi 0
        [5.0, 4.0, 0.0, 0.0, -1.0, 0.0],            # straight down onto the cuboid's top face (y = 1.5)
        [5.0 + 3.0 * math.cos(a), 1.0, -3.0 * math.sin(a), -math.cos(a), 0.0, math.sin(a)],   # onto its +x face
        [-3.0, 1.0, 0.0, 2.0, 0.0, 0.0],            # as the first, but max_toi stops short
        [0.0, 5.0, 0.0, 1.0, 0.0, 0.0],             # misses everything
    ], np.float32)
    max_toi = np.array([3, 10, 10, 10, 1.2, 10], np.float32)   # ray 0 stops before the cuboid (toi 3.75)
    got = w.rays(rays, max_toi)
    want = [(0, 0, 1.25, -1, 0, 0), (1, 0, 0.0, 0, 0, 0), (2, 1, 2.5, 0, 1, 0),
            (3, 1, 2.0, math.cos(a), 0, -math.sin(a))]
    assert len(got) == len(want), got
    for g, e in zip(got, want):
        assert int(g[0]) == e[0] and int(g[1]) == e[1]
        np.testing.assert_allclose(g[2:], e[2:], atol=2e-6)
    pts = np.array([[0.0, 1.4, 0.0], [0.0, 1.6, 0.0], [5.0 + 0.9 * math.cos(a), 1.0, -0.9 * math.sin(a)],
                    [5.0, 1.0, 0.3]], np.float32)
    np.testing.assert_array_equal(w.points(pts), [[0, 0], [2, 1]])
    boxes = np.array([[-1, 0, -1, 1, 2, 1], [2, 0, -1, 3, 2, 1], [3.5, 0, -1, 4.5, 2, 1]], np.float32)
    np.testing.assert_array_equal(w.aabb_query(boxes), [[0, 0], [2, 1]])


def _landing_events(backend):
    # A ball dropped onto the ground: one Started event on the step it first
    # touches (within the prediction distance), none while it rests, and a
    # Stopped event on the step after it is thrown upward.
    sc = scenes.single_body(shape=abi.SHAPE_BALL, params=(0.5, 0, 0), position=(0, 0.8, 0))
    w = _world(backend, sc, events=True)
    seen = []
    for k in range(40):
        w.step(1)
        for e in w.contact_events():
            seen.append((k, int(e[0]), int(e[1]), int(e[2])))
    assert [s[1:] for s in seen] == [(0, 1, 0)], seen
    assert seen[0][0] > 0
    b = sc.bodies.copy()
    pos = w.bodies()["position"]
    b["position"] = pos
    b["velocity"][1] = (0.0, 8.0, 0.0, 0.0, 0.0, 0.0)
    w.upsert_bodies(sc.body_handles[1:], b[1:])
    stops = []
    for k in range(5):
        w.step(1)
        stops += [tuple(int(x) for x in e) for e in w.contact_events()]
    assert stops == [(0, 1, 1)], stops


def test_query_known_answers_oracle():
    _known_answers("oracle")


def test_contact_events_oracle():
    _landing_events("oracle")


@pytest.mark.gpu
def test_query_known_answers_gpu(gpu_lib):
    _known_answers("gpu")


@pytest.mark.gpu
def test_contact_events_gpu(gpu_lib):
    _landing_events("gpu")


@pytest.mark.gpu
def test_random_queries_match_oracle(gpu_lib):
    from nphysics_gb300.world import GpuWorld
    sc = scenes.random_cluster(n=300, seed=12, extent=6.0, capsules=True)
    g = GpuWorld.for_scene(sc, sc.params())
    o = OracleWorld(sc.params(), sc.gravity, precision=32, order=ORDER_COLOUR)
    o.load_scene(sc)
    g.step(20)
    o.step(20)
    np.testing.assert_array_equal(g.bodies()["position"], o.bodies()["position"])
    rng = np.random.default_rng(3)
    n = 2000
    org = rng.uniform(-8, 8, (n, 3)).astype(np.float32)
    org[:, 1] = rng.uniform(-1, 14, n)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    rays = np.concatenate([org, d], axis=1)
    max_toi = rng.uniform(0.5, 20, n).astype(np.float32)
    gr, orr = g.rays(rays, max_toi), o.rays(rays, max_toi)
    assert len(gr) > 500
    np.testing.assert_array_equal(gr[:, :2], orr[:, :2])
    np.testing.assert_allclose(gr[:, 2:], orr[:, 2:], rtol=1e-5, atol=1e-5)
    pts = np.concatenate([rng.uniform(-7, 7, (n, 1)), rng.uniform(-1, 13, (n, 1)), rng.uniform(-7, 7, (n, 1))],
                         axis=1).astype(np.float32)
    gp = g.points(pts)
    assert len(gp) > 100
    np.testing.assert_array_equal(gp, o.points(pts))
    lo = pts - rng.uniform(0, 1.5, (n, 3)).astype(np.float32)
    boxes = np.concatenate([lo, lo + rng.uniform(0, 3, (n, 3)).astype(np.float32)], axis=1)
    gb = g.aabb_query(boxes)
    assert len(gb) > 1000
    np.testing.assert_array_equal(gb, o.aabb_query(boxes))


@pytest.mark.gpu
@pytest.mark.parametrize("sched", [abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS])
def test_pile_events_match_oracle(gpu_lib, sched):
    # A falling batch of small piles: every step's events equal the oracle's,
    # and a world filter keeps each query to one world.
    from nphysics_gb300.world import GpuWorld
    sc = scenes.batched_worlds(n_worlds=6, seed=3, lo=8, hi=120)
    p = sc.params()
    p.solver_schedule = sched
    g = GpuWorld.for_scene(sc, p)
    o = OracleWorld(p, sc.gravity, precision=32, order=ORDER_COLOUR)
    o.load_scene(sc)
    g.enable_contact_events(1 << 16)
    o.enable_contact_events()
    total = 0
    for _ in range(60):
        g.step(1)
        o.step(1)
        ge, oe = g.contact_events(), o.contact_events()
        np.testing.assert_array_equal(ge, oe)
        total += len(ge)
    assert total > 100
    box = np.array([[-50, -5, -50, 50, 50, 50]], np.float32)
    for wd in (0, 3):
        hits = g.aabb_query(box, world=wd)
        np.testing.assert_array_equal(hits, o.aabb_query(box, world=wd))
        bodies_of = sc.colliders["body"]["index"][hits[:, 1]]
        assert (sc.bodies["world"][bodies_of] == wd).all()

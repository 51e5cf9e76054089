"""Known-answer tests of the contact manifolds and the contact re-evaluation.

Each case is a pair of shapes placed so that the exact contact set follows
from the geometry alone: box faces overlapping in a known rectangle, a ball
on a rotated box face, two balls, two boxes touching edge to edge across a
known pair of edges, a box standing on one vertex. The expected points,
normal and depth are computed here from the placement, not taken from any
implementation, and every case runs through the oracle (CPU) and through the
GPU step (the -m gpu twin of each test), so a mistake shared by both would
still fail here. The step runs with gravity off, zero velocities and no
solver iterations, so the contacts reported after it are those of the placed
poses. Conventions (ncollide3d's TrackedContact): world1 lies on collider 1,
world2 on collider 2, the normal points from 1 to 2 and depth > 0 is
penetration, so world1 - world2 = depth * normal.

The position solver's contact re-evaluation (ContactKinematic::contact,
driven at src/solver/nonlinear_sor_prox.rs:221-229, with clamp_rhs at
:296-309) is pinned by its recurrence: a ball resting into the ground, or two
balls overlapping, is pushed apart along the normal by
-max((-depth + allowed_linear_error) * erp, -max_linear_correction) per
iteration, and each iteration re-evaluates the depth at the moved poses.
"""
import math

import numpy as np
import pytest

from nphysics_gb300 import abi, scenes
from oracle.oracle_py import ORDER_COLOUR, OracleWorld

DEPTH = 0.05
TOL = 2e-6        # absolute, on coordinates of order 1 (f32 geometry)


def _quat_from_matrix(R):
    """(i, j, k, w) of a rotation matrix (Shepperd's method)."""
    t = np.trace(R)
    if t > 0:
        s = math.sqrt(t + 1.0) * 2
        q = ((R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s, 0.25 * s)
    else:
        i = int(np.argmax(np.diag(R)))
        j, k = (i + 1) % 3, (i + 2) % 3
        s = math.sqrt(1.0 + R[i, i] - R[j, j] - R[k, k]) * 2
        v = [0.0, 0.0, 0.0]
        v[i] = 0.25 * s
        v[j] = (R[j, i] + R[i, j]) / s
        v[k] = (R[k, i] + R[i, k]) / s
        q = (v[0], v[1], v[2], (R[k, j] - R[j, k]) / s)
    return np.array(q, np.float64)


def _rotation_taking(a, b):
    """The rotation matrix turning unit vector a onto unit vector b."""
    a, b = np.asarray(a, float), np.asarray(b, float)
    v = np.cross(a, b)
    c = float(a @ b)
    K = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
    return np.eye(3) + K + K @ K / (1.0 + c)


def two_shapes(shape1, params1, pose1, shape2, params2, pose2, dynamic1=False, dynamic2=True):
    """Collider 0 on body 0 (a static rigid body at pose1 unless dynamic1),
    collider 1 on body 1."""
    b = scenes.body_descs(2)
    for i, dyn in ((0, dynamic1), (1, dynamic2)):
        if not dyn:
            b["status"][i] = abi.BODY_STATIC
    b["position"][0] = pose1
    b["position"][1] = pose2
    c = np.concatenate([scenes.collider_descs(1, 0, shape1, params1, density=1.0),
                        scenes.collider_descs(1, 1, shape2, params2, density=1.0)])
    return scenes.Scene("manifold known answer", b, c, gravity=(0.0, 0.0, 0.0))


def pose(t, R=None):
    q = _quat_from_matrix(R) if R is not None else np.array([0.0, 0.0, 0.0, 1.0])
    return tuple(t) + tuple(q)


def step_once(backend, scene, velocity_iterations=0, position_iterations=0):
    p = scene.params()
    p.max_velocity_iterations = velocity_iterations
    p.max_position_iterations = position_iterations
    if backend == "gpu":
        from nphysics_gb300.world import GpuWorld
        w = GpuWorld.for_scene(scene, p)
    else:
        w = OracleWorld(p, scene.gravity, precision=32, order=ORDER_COLOUR)
        w.load_scene(scene)
    w.step(1)
    return w


def check_manifold(backend, scene, want_world1, want_world2, normal, depth):
    c = step_once(backend, scene).contacts()
    assert len(c["depth"]) == len(want_world1), c["depth"]
    assert (c["collider1"] == 0).all() and (c["collider2"] == 1).all()
    order = np.lexsort(np.asarray(c["world1"], np.float64).T[::-1])
    want1 = np.asarray(want_world1, np.float64)
    want2 = np.asarray(want_world2, np.float64)
    worder = np.lexsort(want1.T[::-1])
    np.testing.assert_allclose(np.asarray(c["world1"], np.float64)[order], want1[worder], atol=TOL)
    np.testing.assert_allclose(np.asarray(c["world2"], np.float64)[order], want2[worder], atol=TOL)
    np.testing.assert_allclose(np.asarray(c["normal"], np.float64), np.tile(normal, (len(want1), 1)), atol=TOL)
    np.testing.assert_allclose(np.asarray(c["depth"], np.float64), depth, atol=TOL)


# ---------------------------------------------------------------- the cases
def case_face_face():
    # A: half extents 1 at the origin; B: half extents 0.5, its bottom face
    # 0.05 below A's top face and offset so that only [0.3, 1] x [-0.2, 0.8]
    # of it lies over A: four contacts at that rectangle's corners.
    sc = two_shapes(abi.SHAPE_CUBOID, (1, 1, 1), pose((0, 0, 0)), abi.SHAPE_CUBOID, (0.5, 0.5, 0.5),
                    pose((0.8, 1.5 - DEPTH, 0.3)))
    xz = [(0.3, -0.2), (0.3, 0.8), (1.0, 0.8), (1.0, -0.2)]
    return sc, [(x, 1.0, z) for x, z in xz], [(x, 1.0 - DEPTH, z) for x, z in xz], (0, 1, 0), DEPTH


def case_box_on_ground():
    # The pyramid's box on the ground cuboid: four corners.
    sc = two_shapes(abi.SHAPE_CUBOID, (50, 1, 50), pose((0, -1, 0)), abi.SHAPE_CUBOID, (0.5, 0.5, 0.5),
                    pose((2.0, 0.5 - DEPTH, -3.0)))
    xz = [(1.5, -3.5), (1.5, -2.5), (2.5, -2.5), (2.5, -3.5)]
    return sc, [(x, 0.0, z) for x, z in xz], [(x, -DEPTH, z) for x, z in xz], (0, 1, 0), DEPTH


def case_ball_on_rotated_box():
    # A box turned 30 degrees about y; a ball of radius 0.5 over its top face
    # at box-local (0.3, ., -0.2), 0.05 into it.
    a = math.radians(30)
    R = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
    local = np.array([0.3, 1.0, -0.2])
    top = R @ local
    centre = top + np.array([0, 0.5 - DEPTH, 0])
    sc = two_shapes(abi.SHAPE_CUBOID, (1, 1, 1), pose((0, 0, 0), R), abi.SHAPE_BALL, (0.5, 0, 0), pose(centre))
    return sc, [top], [centre - np.array([0, 0.5, 0])], (0, 1, 0), DEPTH


def case_ball_ball():
    # Radii 0.4 and 0.7 along a skew direction, 0.05 closer than touching.
    n = np.array([2.0, -1.0, 2.0]) / 3.0
    c1 = np.array([0.1, 2.0, -0.3])
    c2 = c1 + n * (0.4 + 0.7 - DEPTH)
    sc = two_shapes(abi.SHAPE_BALL, (0.4, 0, 0), pose(c1), abi.SHAPE_BALL, (0.7, 0, 0), pose(c2))
    return sc, [c1 + 0.4 * n], [c2 - 0.7 * n], n, DEPTH


def case_edge_edge():
    # A: half extents 1 at the origin; its edge (t, 1, 1) where the top and
    # front faces meet. B: a cube of half extent 0.5 turned so that one of its
    # edges runs along (0, 1, -1)/sqrt2, across A's edge, and its two faces at
    # that edge look down the bisector -n, n = (0, 1, 1)/sqrt2. The edges
    # cross at P = (0, 1, 1) on A and P - 0.05 n on B.
    n = np.array([0.0, 1.0, 1.0]) / math.sqrt(2.0)
    U = np.stack([[1, 0, 0], np.array([0, 1, 1]) / math.sqrt(2), np.array([0, -1, 1]) / math.sqrt(2)], axis=1)
    V = np.stack([np.array([0, 1, -1]) / math.sqrt(2), n, [1, 0, 0]], axis=1)
    R = V @ U.T
    P = np.array([0.0, 1.0, 1.0])
    centre = P + n * (0.5 * math.sqrt(2.0) - DEPTH)
    sc = two_shapes(abi.SHAPE_CUBOID, (1, 1, 1), pose((0, 0, 0)), abi.SHAPE_CUBOID, (0.5, 0.5, 0.5),
                    pose(centre, R))
    return sc, [P], [P - DEPTH * n], n, DEPTH


def case_vertex_face():
    # B stands on one vertex: its local corner (-h, -h, -h) turned straight
    # down, 0.05 into A's top face at (0.2, ., -0.4).
    h = 0.5
    R = _rotation_taking(-np.ones(3) / math.sqrt(3.0), [0, -1, 0])
    vertex = np.array([0.2, 1.0 - DEPTH, -0.4])
    centre = vertex + np.array([0, h * math.sqrt(3.0), 0])
    sc = two_shapes(abi.SHAPE_CUBOID, (1, 1, 1), pose((0, 0, 0)), abi.SHAPE_CUBOID, (h, h, h), pose(centre, R))
    return sc, [vertex + np.array([0, DEPTH, 0])], [vertex], (0, 1, 0), DEPTH


def _rot_z90():
    # Turns the capsule's axis (local y) onto world x.
    return np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])


def case_capsule_lying_on_box():
    # A capsule (radius 0.3, half height 0.8) lying along x on the ground
    # cuboid, 0.05 into it: one contact under each end.
    r, hh = 0.3, 0.8
    centre = np.array([1.0, r - DEPTH, -2.0])
    sc = two_shapes(abi.SHAPE_CUBOID, (50, 1, 50), pose((0, -1, 0)), abi.SHAPE_CAPSULE, (r, hh, 0),
                    pose(centre, _rot_z90()))
    ends = [centre + np.array([-hh, 0, 0]), centre + np.array([hh, 0, 0])]
    return (sc, [e - np.array([0, e[1], 0]) for e in ends], [e - np.array([0, r, 0]) for e in ends], (0, 1, 0),
            DEPTH)


def case_capsule_standing_on_box():
    # Upright on the ground: one contact under its lower end.
    r, hh = 0.3, 0.8
    centre = np.array([0.5, hh + r - DEPTH, 0.2])
    sc = two_shapes(abi.SHAPE_CUBOID, (50, 1, 50), pose((0, -1, 0)), abi.SHAPE_CAPSULE, (r, hh, 0), pose(centre))
    low = centre - np.array([0, hh, 0])
    return sc, [low * np.array([1, 0, 1])], [low - np.array([0, r, 0])], (0, 1, 0), DEPTH


def case_capsule_along_box_edge():
    # A capsule along z lying on the top +x edge of a box (half 1), longer
    # than the edge: a contact at each end of the edge (the edge's vertices
    # against the axis), the normal from the edge toward the axis.
    r, hh = 0.25, 1.5
    n = np.array([1.0, 1.0, 0.0]) / math.sqrt(2.0)
    R = np.array([[1.0, 0.0, 0.0], [0.0, 0.0, -1.0], [0.0, 1.0, 0.0]])   # local y onto world z
    centre = np.array([1.0, 1.0, 0.3]) + n * (r - DEPTH)
    sc = two_shapes(abi.SHAPE_CUBOID, (1, 1, 1), pose((0, 0, 0)), abi.SHAPE_CAPSULE, (r, hh, 0), pose(centre, R))
    ends = [np.array([1.0, 1.0, -1.0]), np.array([1.0, 1.0, 1.0])]
    return sc, ends, [e - n * DEPTH for e in ends], n, DEPTH


def case_capsule_across_box_edge():
    # A horizontal capsule along x over the top +x edge of a box (half 1):
    # its inner end rests on the top face, its axis crosses the edge; the
    # face clipping gives the end's contact and one at the edge.
    r, hh = 0.25, 0.6
    centre = np.array([0.9, 1.0 + r - DEPTH, 0.2])
    sc = two_shapes(abi.SHAPE_CUBOID, (1, 1, 1), pose((0, 0, 0)), abi.SHAPE_CAPSULE, (r, hh, 0),
                    pose(centre, _rot_z90()))
    inner = centre - np.array([hh, 0, 0])
    at_edge = np.array([1.0, centre[1], centre[2]])
    return (sc, [np.array([inner[0], 1.0, inner[2]]), np.array([1.0, 1.0, centre[2]])],
            [inner - np.array([0, r, 0]), at_edge - np.array([0, r, 0])], (0, 1, 0), DEPTH)


def case_ball_on_capsule():
    # A ball resting on the middle of a horizontal capsule.
    r, hh, rb = 0.3, 0.8, 0.4
    c0 = np.array([0.0, 2.0, 0.0])
    cb = c0 + np.array([0.2, r + rb - DEPTH, 0.0])
    sc = two_shapes(abi.SHAPE_CAPSULE, (r, hh, 0), pose(c0, _rot_z90()), abi.SHAPE_BALL, (rb, 0, 0), pose(cb))
    axis_pt = np.array([0.2, 2.0, 0.0])
    return sc, [axis_pt + np.array([0, r, 0])], [cb - np.array([0, rb, 0])], (0, 1, 0), DEPTH


def case_capsules_parallel():
    # Two parallel horizontal capsules, one on the other, overlapping over
    # x in [-0.2, 0.8]: a contact at each end of the overlap.
    r, hh = 0.3, 0.8
    c0 = np.array([0.0, 2.0, 0.0])
    c1 = c0 + np.array([1.0, 2 * r - DEPTH, 0.0])
    sc = two_shapes(abi.SHAPE_CAPSULE, (r, hh, 0), pose(c0, _rot_z90()), abi.SHAPE_CAPSULE, (r, hh, 0),
                    pose(c1, _rot_z90()))
    xs = [0.2, 0.8]
    return (sc, [np.array([x, 2.0 + r, 0.0]) for x in xs], [np.array([x, c1[1] - r, 0.0]) for x in xs], (0, 1, 0),
            DEPTH)


def case_capsules_crossing():
    # A capsule along x under one along z: one contact at the crossing.
    r, hh = 0.3, 0.8
    c0 = np.array([0.1, 2.0, -0.2])
    Rz = np.array([[1.0, 0.0, 0.0], [0.0, 0.0, -1.0], [0.0, 1.0, 0.0]])
    c1 = c0 + np.array([0.3, 2 * r - DEPTH, 0.4])
    sc = two_shapes(abi.SHAPE_CAPSULE, (r, hh, 0), pose(c0, _rot_z90()), abi.SHAPE_CAPSULE, (r, hh, 0), pose(c1, Rz))
    x = np.array([c1[0], c0[1], c0[2]])
    return sc, [x + np.array([0, r, 0])], [np.array([c1[0], c1[1] - r, c0[2]])], (0, 1, 0), DEPTH


CASES = {
    "capsule_lying_on_box": case_capsule_lying_on_box,
    "capsule_standing_on_box": case_capsule_standing_on_box,
    "capsule_along_box_edge": case_capsule_along_box_edge,
    "capsule_across_box_edge": case_capsule_across_box_edge,
    "ball_on_capsule": case_ball_on_capsule,
    "capsules_parallel": case_capsules_parallel,
    "capsules_crossing": case_capsules_crossing,
    "face_face": case_face_face,
    "box_on_ground": case_box_on_ground,
    "ball_on_rotated_box": case_ball_on_rotated_box,
    "ball_ball": case_ball_ball,
    "edge_edge": case_edge_edge,
    "vertex_face": case_vertex_face,
}


def _manifold(backend, name):
    sc, w1, w2, n, d = CASES[name]()
    check_manifold(backend, sc, w1, w2, np.asarray(n, np.float64), d)


def _position_recurrence(depth, iterations, erp=0.2, allowed=0.001, max_corr=0.2):
    """Total push along the normal after `iterations` position iterations of
    one contact whose depth is re-evaluated after every push."""
    total = 0.0
    for _ in range(iterations):
        rhs = max((-depth + allowed) * erp, -max_corr)
        if rhs >= 0.0:
            break
        total -= rhs
        depth += rhs
    return total


# The position constraint's contact kinematic is dilated by both colliders'
# margins (build_position_constraint, src/solver/signorini_model.rs:153-197),
# so the depth it re-evaluates is the shapes' overlap plus 2 x 0.01.
MARGINS = 2 * scenes.DEFAULT_MARGIN


def _reevaluation_ball_on_ground(backend):
    d = 0.3
    sc = two_shapes(abi.SHAPE_CUBOID, (50, 1, 50), pose((0, -1, 0)), abi.SHAPE_BALL, (0.5, 0, 0),
                    pose((1.0, 0.5 - d, 2.0)))
    w = step_once(backend, sc, position_iterations=3)
    y = float(w.bodies()["position"][1, 1])
    assert abs(y - (0.5 - d + _position_recurrence(d + MARGINS, 3))) < 2e-6


def _reevaluation_two_balls(backend):
    # Equal balls, both dynamic: each moves half of every push.
    d = 0.4
    n = np.array([1.0, 2.0, -2.0]) / 3.0
    c1 = np.array([0.0, 3.0, 0.0])
    c2 = c1 + n * (1.0 - d)
    sc = two_shapes(abi.SHAPE_BALL, (0.5, 0, 0), pose(c1), abi.SHAPE_BALL, (0.5, 0, 0), pose(c2), dynamic1=True)
    w = step_once(backend, sc, position_iterations=3)
    pos = w.bodies()["position"][:, :3].astype(np.float64)
    push = _position_recurrence(d + MARGINS, 3)
    np.testing.assert_allclose(pos[0], c1 - 0.5 * push * n, atol=3e-6)
    np.testing.assert_allclose(pos[1], c2 + 0.5 * push * n, atol=3e-6)


@pytest.mark.parametrize("name", sorted(CASES))
def test_manifold_oracle(name):
    _manifold("oracle", name)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_manifold_gpu(gpu_lib, name):
    _manifold("gpu", name)


def test_contact_reevaluation_oracle():
    _reevaluation_ball_on_ground("oracle")
    _reevaluation_two_balls("oracle")


@pytest.mark.gpu
def test_contact_reevaluation_gpu(gpu_lib):
    _reevaluation_ball_on_ground("gpu")
    _reevaluation_two_balls("gpu")

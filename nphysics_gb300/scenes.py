"""Scene builders: the rigid-body scenes the step is measured and checked on.

Each builder returns a `Scene`: structured numpy arrays laid out exactly as
`npgpu_body_desc` / `npgpu_collider_desc` (include/npgpu.h), plus handles.
Defaults follow RigidBodyDesc::new (src/object/rigid_body.rs:974-995),
ColliderDesc::new (src/object/collider.rs:455-479) and BasicMaterial::default
(src/material/basic_material.rs:59-63). Recipes follow examples3d/pyramid3.rs,
balls3.rs and wall3.rs, scaled to the benchmark configurations.
"""
import math

import numpy as np

from . import abi

BODY_DTYPE = np.dtype(abi.BodyDesc)
COLLIDER_DTYPE = np.dtype(abi.ColliderDesc)
HANDLE_DTYPE = np.dtype(abi.Handle)
JOINT_DTYPE = np.dtype(abi.JointDesc)
DEFAULT_SLEEP_THRESHOLD = 0.01   # ActivationStatus::default_threshold (src/object/body.rs:72-74)
DEFAULT_MARGIN = 0.01
DEFAULT_LINEAR_PREDICTION = 0.001
DEFAULT_ANGULAR_PREDICTION = math.pi / 180.0 * 5.0


class Scene:
    def __init__(self, name, bodies, colliders, gravity=(0.0, -9.81, 0.0), dt=1.0 / 60.0, steps=1, info=None):
        self.name = name
        self.bodies = bodies
        self.colliders = colliders
        self.body_handles = make_handles(len(bodies))
        self.collider_handles = make_handles(len(colliders))
        self.joints = np.zeros(0, JOINT_DTYPE)
        self.joint_handles = make_handles(0)
        self.gravity = tuple(float(g) for g in gravity)
        self.dt = float(dt)
        self.steps = int(steps)
        self.info = dict(info or {})

    @property
    def num_dynamic(self):
        return int(np.count_nonzero(self.bodies["status"] == abi.BODY_DYNAMIC))

    def params(self):
        p = abi.default_params()
        p.dt = self.dt
        return p


def joint_descs(n):
    """n joint descriptions with identity frames and unbreakable limits."""
    j = np.zeros(n, JOINT_DTYPE)
    j["frame1"][:, 3] = 1.0
    j["frame2"][:, 3] = 1.0
    j["break_force"] = abi.FLT_MAX
    j["break_torque"] = abi.FLT_MAX
    j["axis1"][:, 0] = 1.0
    j["axis2"][:, 0] = 1.0
    j["axis3"][:, 0] = 1.0
    return j


def set_joints(scene, joints):
    """Attaches joint descriptions (JOINT_DTYPE) to a scene, with handles 0..n-1."""
    scene.joints = np.ascontiguousarray(joints)
    scene.joint_handles = make_handles(len(joints))
    return scene


def make_handles(n, generation=0):
    h = np.zeros(n, HANDLE_DTYPE)
    h["index"] = np.arange(n, dtype=np.uint64)
    h["generation"] = generation
    return h


def body_descs(n):
    """n copies of RigidBodyDesc::new().build()."""
    b = np.zeros(n, BODY_DTYPE)
    b["position"][:, 6] = 1.0
    b["max_linear_velocity"] = abi.FLT_MAX
    b["max_angular_velocity"] = abi.FLT_MAX
    b["sleep_threshold"] = DEFAULT_SLEEP_THRESHOLD
    b["status"] = abi.BODY_DYNAMIC
    b["kind"] = abi.KIND_RIGID_BODY
    b["flags"] = abi.BODY_GRAVITY | abi.BODY_CAN_SLEEP
    return b


def ground_descs(n):
    """n copies of Ground::new() (src/object/ground.rs:21-27)."""
    b = body_descs(n)
    b["status"] = abi.BODY_STATIC
    b["kind"] = abi.KIND_GROUND
    b["flags"] = 0
    return b


def collider_descs(n, body_index, shape, params, density=0.0, friction=0.5, restitution=0.0):
    c = np.zeros(n, COLLIDER_DTYPE)
    c["body"]["index"] = body_index
    c["body"]["generation"] = 0
    c["position_wrt_body"][:, 6] = 1.0
    c["shape_params"] = params
    c["margin"] = DEFAULT_MARGIN
    c["density"] = density
    c["linear_prediction"] = DEFAULT_LINEAR_PREDICTION
    c["angular_prediction"] = DEFAULT_ANGULAR_PREDICTION
    c["friction"] = friction
    c["restitution"] = restitution
    c["shape"] = shape
    return c


def uniform_quaternions(rng, n):
    """Uniform random rotations (Shoemake 1992), (i, j, k, w) order."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    q = np.stack([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                  b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)], axis=1)
    return q.astype(np.float32)


def _ground(half=(50.0, 1.0, 50.0), friction=0.5, world=0):
    g = ground_descs(1)
    g["world"] = world
    gc = collider_descs(1, 0, abi.SHAPE_CUBOID, half, density=0.0, friction=friction)
    gc["position_wrt_body"][0, 1] = -half[1]     # top face at y = 0
    return g, gc


def _concat(parts_b, parts_c):
    """Concatenates (bodies, colliders) groups, re-pointing collider parents."""
    bodies, colliders, off = [], [], 0
    for b, c in zip(parts_b, parts_c):
        c = c.copy()
        c["body"]["index"] = c["body"]["index"] + off
        bodies.append(b)
        colliders.append(c)
        off += len(b)
    return np.concatenate(bodies), np.concatenate(colliders)


def pyramid(base=20, half=0.5, friction=0.5):
    """C1: a 2D triangle of cuboids (base 20 -> 210 boxes, half extents 0.5,
    1.0 spacing) on a static 50 x 1 x 50 ground, density 1, friction 0.5."""
    xs, ys = [], []
    for row in range(base):
        for i in range(base - row):
            xs.append(i * 2 * half + row * half - (base - 1) * half)
            ys.append(half + row * 2 * half)
    n = len(xs)
    g, gc = _ground(friction=friction)
    b = body_descs(n)
    b["position"][:, 0] = xs
    b["position"][:, 1] = ys
    c = collider_descs(n, np.arange(n), abi.SHAPE_CUBOID, (half, half, half), density=1.0, friction=friction)
    bodies, colliders = _concat([g, b], [gc, c])
    return Scene(f"box pyramid (base {base}, {n} cuboids)", bodies, colliders, steps=1000,
                 info={"boxes": n})


def ball_pile(side=32, radius=0.5, spacing=1.2, jitter=0.05, seed=1234, friction=0.3):
    """C2: side^3 balls (radius 0.5) on a 1.2 lattice with U(-0.05, 0.05) jitter,
    dropped on a static 100 x 1 x 100 ground; density 1, friction 0.3."""
    rng = np.random.default_rng(seed)
    n = side ** 3
    i, j, k = np.meshgrid(np.arange(side), np.arange(side), np.arange(side), indexing="ij")
    pos = np.stack([(i.ravel() - (side - 1) / 2) * spacing,
                    1.0 + j.ravel() * spacing,
                    (k.ravel() - (side - 1) / 2) * spacing], axis=1)
    pos += rng.uniform(-jitter, jitter, size=pos.shape)
    g, gc = _ground(half=(100.0, 1.0, 100.0), friction=friction)
    b = body_descs(n)
    b["position"][:, :3] = pos.astype(np.float32)
    c = collider_descs(n, np.arange(n), abi.SHAPE_BALL, (radius, 0, 0), density=1.0, friction=friction)
    bodies, colliders = _concat([g, b], [gc, c])
    return Scene(f"ball pile ({side}^3 = {n} balls)", bodies, colliders, steps=600, info={"balls": n})


def mixed_lattice(n=100_000, seed=1234, friction=0.5, spacing=2.0, footprint=100.0):
    """A lattice-placed mixed pile: n bodies, half balls with radius U(0.2, 0.8) and half cuboids with
    half extents U(0.2, 0.8)^3 and uniform random orientation, density 1,
    friction 0.5, over a 100 x 100 footprint. Bodies sit on a jittered 2.0
    lattice of layers from y = 1 upward so that none overlap at t = 0."""
    rng = np.random.default_rng(seed)
    per_side = int(footprint // spacing)
    per_layer = per_side * per_side
    idx = np.arange(n)
    layer, rem = idx // per_layer, idx % per_layer
    gx, gz = rem % per_side, rem // per_side
    pos = np.stack([(gx - (per_side - 1) / 2) * spacing, 1.0 + layer * spacing,
                    (gz - (per_side - 1) / 2) * spacing], axis=1).astype(np.float64)
    pos += rng.uniform(-0.1, 0.1, size=pos.shape)
    is_ball = rng.permutation(n) < n // 2
    g, gc = _ground(half=(footprint * 0.6, 1.0, footprint * 0.6), friction=friction)
    b = body_descs(n)
    b["position"][:, :3] = pos.astype(np.float32)
    b["position"][:, 3:7] = uniform_quaternions(rng, n)
    shape = np.where(is_ball, abi.SHAPE_BALL, abi.SHAPE_CUBOID).astype(np.uint32)
    params = np.zeros((n, 3), np.float32)
    params[is_ball, 0] = rng.uniform(0.2, 0.8, size=int(is_ball.sum()))
    params[~is_ball] = rng.uniform(0.2, 0.8, size=(int((~is_ball).sum()), 3))
    c = collider_descs(n, np.arange(n), abi.SHAPE_BALL, (0, 0, 0), density=1.0, friction=friction)
    c["shape"] = shape
    c["shape_params"] = params
    bodies, colliders = _concat([g, b], [gc, c])
    return Scene(f"mixed lattice pile ({n} bodies)", bodies, colliders, steps=300, info={"bodies": n})


def _quat_matrices(q):
    """Rotation matrices of unit quaternions in (i, j, k, w) order."""
    x, y, z, w = (q[:, k].astype(np.float64) for k in range(4))
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], axis=1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], axis=1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], axis=1)], axis=1)


def _close_pairs(pos_q, rad_q, pos_o, rad_o, gap):
    """Pairs (q, o) of a query set and another set of bodies whose bounding
    spheres come within `gap` of each other (k-d tree range search)."""
    from scipy.spatial import cKDTree
    r = float(rad_q.max()) + float(rad_o.max()) + gap
    m = cKDTree(pos_q).sparse_distance_matrix(cKDTree(pos_o), r, output_type="ndarray")
    q, o = m["i"].astype(np.int64), m["j"].astype(np.int64)
    near = m["v"] < rad_q[q] + rad_o[o] + gap
    return q[near], o[near]


def _shapes_overlap(i, j, pos, rot, is_ball, half, gap):
    """Exact overlap test, inflated by `gap`, of the (ball or cuboid) shapes of
    bodies i and j: distance of centres for two balls, the closest point of the
    box for a ball and a box, the 15 separating axes for two boxes."""
    out = np.zeros(len(i), bool)
    bb = is_ball[i] & is_ball[j]
    out[bb] = np.linalg.norm(pos[i[bb]] - pos[j[bb]], axis=1) < half[i[bb], 0] + half[j[bb], 0] + gap
    mixed = is_ball[i] != is_ball[j]
    if mixed.any():
        b = np.where(is_ball[i[mixed]], i[mixed], j[mixed])
        x = np.where(is_ball[i[mixed]], j[mixed], i[mixed])
        local = np.einsum("nji,nj->ni", rot[x], pos[b] - pos[x])
        closest = np.clip(local, -half[x], half[x])
        out[mixed] = np.linalg.norm(local - closest, axis=1) < half[b, 0] + gap
    xx = ~is_ball[i] & ~is_ball[j]
    if xx.any():
        a, b = i[xx], j[xx]
        Ra, Rb, ha, hb = rot[a], rot[b], half[a], half[b]
        d = pos[b] - pos[a]
        axes = [Ra[:, :, k] for k in range(3)] + [Rb[:, :, k] for k in range(3)]
        axes += [np.cross(Ra[:, :, p], Rb[:, :, q]) for p in range(3) for q in range(3)]
        sep = np.zeros(len(a), bool)
        for L in axes:
            ln = np.linalg.norm(L, axis=1)
            ok = ln > 1e-9
            ra = sum(ha[:, k] * np.abs(np.einsum("ni,ni->n", Ra[:, :, k], L)) for k in range(3))
            rb = sum(hb[:, k] * np.abs(np.einsum("ni,ni->n", Rb[:, :, k], L)) for k in range(3))
            sep |= ok & (np.abs(np.einsum("ni,ni->n", d, L)) > ra + rb + gap * ln)
        out[xx] = ~sep
    return out


def mixed_pile(n=100_000, seed=1234, friction=0.5, footprint=100.0, heights=(1.0, 60.0), gap=0.05):
    """C3: n bodies, half balls with radius U(0.2, 0.8) and half cuboids with
    half extents U(0.2, 0.8)^3 and uniform random orientation (Shoemake),
    density 1, friction 0.5, dropped from centre heights U(1, 60) over a
    100 x 100 footprint (x, z in U(-50, 50)) onto a static ground.

    Initial overlaps are resolved by seeded rejection: the draws are made in
    body order from one generator, then, pass after pass, every body that
    overlaps an earlier one (exact ball / cuboid tests, inflated by `gap`) or
    reaches below the ground's top face draws a new position from the same
    distribution, until no body overlaps. Shapes and orientations are kept."""
    rng = np.random.default_rng(seed)
    is_ball = rng.permutation(n) < n // 2
    half = np.zeros((n, 3), np.float32)
    half[is_ball, 0] = rng.uniform(0.2, 0.8, size=int(is_ball.sum()))
    half[~is_ball] = rng.uniform(0.2, 0.8, size=(int((~is_ball).sum()), 3))
    quat = uniform_quaternions(rng, n)
    quat[is_ball] = (0.0, 0.0, 0.0, 1.0)
    lo = -footprint / 2

    def draw(k):
        p = np.stack([rng.uniform(lo, -lo, k), rng.uniform(heights[0], heights[1], k), rng.uniform(lo, -lo, k)],
                     axis=1)
        return p.astype(np.float32).astype(np.float64)

    pos = draw(n)
    rot = _quat_matrices(quat)
    h64 = half.astype(np.float64)
    radius = np.where(is_ball, h64[:, 0], np.linalg.norm(h64, axis=1))
    # Lowest point of each shape above the ground's top face (y = 0).
    reach = np.where(is_ball, h64[:, 0], np.einsum("nk,nk->n", np.abs(rot[:, 1, :]), h64))
    # Seeded random sequential addition in body order: a pending body is
    # placed once it overlaps neither a placed body nor an earlier pending one;
    # one that overlaps a placed body or the ground moves to the first of a
    # batch of fresh draws that is clear of every other body (the batch's last
    # draw when none is).
    pending = np.ones(n, bool)
    passes = 0
    while pending.any():
        q_idx = np.nonzero(pending)[0]
        q, o = _close_pairs(pos[q_idx], radius[q_idx], pos, radius, gap)
        q = q_idx[q]
        keep = q != o
        q, o = q[keep], o[keep]
        hit = _shapes_overlap(q, o, pos, rot, is_ball, h64, gap)
        q, o = q[hit], o[hit]
        redraw = np.zeros(n, bool)
        wait = np.zeros(n, bool)
        redraw[q[~pending[o]]] = True
        wait[q[pending[o] & (o < q)]] = True
        redraw |= pending & (pos[:, 1] - reach < gap)
        pending &= redraw | wait
        movers = np.nonzero(redraw)[0]
        if len(movers):
            m = int(max(1, min(64, 65536 // len(movers))))
            cand = draw(len(movers) * m)
            owner = np.repeat(movers, m)
            cq, co = _close_pairs(cand, radius[owner], pos, radius, gap)
            keep = co != owner[cq]
            cq, co = cq[keep], co[keep]
            ext = np.concatenate([pos, cand])
            ov = _shapes_overlap(cq + n, co, ext, np.concatenate([rot, rot[owner]]),
                                 np.concatenate([is_ball, is_ball[owner]]), np.concatenate([h64, h64[owner]]), gap)
            blocked = np.zeros(len(cand), bool)
            blocked[cq[ov]] = True
            blocked |= cand[:, 1] - reach[owner] < gap
            free = ~blocked.reshape(len(movers), m)
            pick = np.where(free.any(axis=1), free.argmax(axis=1), m - 1)
            pos[movers] = cand.reshape(len(movers), m, 3)[np.arange(len(movers)), pick]
        passes += 1
        if passes > 1000:
            raise RuntimeError("mixed_pile: overlaps not resolved in 1000 passes")
    g, gc = _ground(half=(footprint * 0.8, 1.0, footprint * 0.8), friction=friction)
    b = body_descs(n)
    b["position"][:, :3] = pos.astype(np.float32)
    b["position"][:, 3:7] = quat
    c = collider_descs(n, np.arange(n), abi.SHAPE_BALL, (0, 0, 0), density=1.0, friction=friction)
    c["shape"] = np.where(is_ball, abi.SHAPE_BALL, abi.SHAPE_CUBOID).astype(np.uint32)
    c["shape_params"] = half
    bodies, colliders = _concat([g, b], [gc, c])
    return Scene(f"mixed pile ({n} bodies)", bodies, colliders, steps=300,
                 info={"bodies": n, "placement_passes": passes})


def batched_worlds(n_worlds=4096, seed=1234, lo=16, hi=2048, worlds=None):
    """C4: independent worlds with body counts log-uniform in [16, 2048], each
    a scaled-down ball pile or a box stack of height U(3, 15) on its own ground.
    Worlds share space; the world index keeps them apart.

    `worlds` (a range, default all) builds only those worlds of the batch, with
    the same bodies as in the whole batch, renumbered from world 0: the shard
    of one rank when the batch is split across GPUs."""
    rng = np.random.default_rng(seed)
    counts = np.round(np.exp(rng.uniform(math.log(lo), math.log(hi), size=n_worlds))).astype(int)
    kinds = rng.random(n_worlds) < 0.5
    worlds = range(n_worlds) if worlds is None else worlds
    parts_b, parts_c = [], []
    for local, w in enumerate(worlds):
        wr = np.random.default_rng([seed, w])       # the world's own draws
        nb = int(counts[w])
        g, gc = _ground(half=(60.0, 1.0, 60.0), world=local)
        b = body_descs(nb)
        b["world"] = local
        if kinds[w]:
            side = int(math.ceil(nb ** (1.0 / 3.0)))
            idx = np.arange(nb)
            i, j, k = idx % side, (idx // side) % side, idx // (side * side)
            pos = np.stack([(i - (side - 1) / 2) * 1.2, 1.0 + k * 1.2, (j - (side - 1) / 2) * 1.2], axis=1)
            pos += wr.uniform(-0.05, 0.05, size=pos.shape)
            c = collider_descs(nb, np.arange(nb), abi.SHAPE_BALL, (0.5, 0, 0), density=1.0, friction=0.3)
        else:
            height = int(wr.integers(3, 16))
            cols = int(math.ceil(nb / height))
            cs = int(math.ceil(math.sqrt(cols)))
            idx = np.arange(nb)
            col, lev = idx // height, idx % height
            pos = np.stack([(col % cs - (cs - 1) / 2) * 1.5, 0.5 + lev * 1.0, (col // cs - (cs - 1) / 2) * 1.5],
                           axis=1)
            c = collider_descs(nb, np.arange(nb), abi.SHAPE_CUBOID, (0.5, 0.5, 0.5), density=1.0, friction=0.5)
        b["position"][:, :3] = pos.astype(np.float32)
        parts_b += [g, b]
        parts_c += [gc, c]
    bodies, colliders = _concat(parts_b, parts_c)
    return Scene(f"{len(worlds)} of {n_worlds} batched worlds", bodies, colliders, steps=100,
                 info={"worlds": len(worlds), "bodies": int(counts[list(worlds)].sum())})


def brick_walls(n_walls=256, width=50, height=40, balls=64, seed=1234, ccd=False):
    """C5: walls of width x height bricks (half extents 0.5 x 0.25 x 0.25,
    running bond) each struck by `balls` balls of radius 0.4, density 10, at
    U(20, 40) m/s with a +-5 degree direction jitter; friction 0.6, dt 1/120.
    With `ccd` the balls' colliders have CCD enabled."""
    rng = np.random.default_rng(seed)
    parts_b, parts_c = [], []
    for w in range(n_walls):
        g, gc = _ground(half=(60.0, 1.0, 60.0), friction=0.6, world=w)
        xs, ys = [], []
        for r in range(height):
            off = 0.5 if r % 2 else 0.0
            for i in range(width):
                xs.append((i - width / 2) * 1.0 + off)
                ys.append(0.25 + r * 0.5)
        nb = len(xs)
        b = body_descs(nb)
        b["world"] = w
        b["position"][:, 0] = xs
        b["position"][:, 1] = ys
        c = collider_descs(nb, np.arange(nb), abi.SHAPE_CUBOID, (0.5, 0.25, 0.25), density=1.0, friction=0.6)
        bb = body_descs(balls)
        bb["world"] = w
        start = np.stack([rng.uniform(-width / 2, width / 2, balls), rng.uniform(1.0, height * 0.5, balls),
                          np.full(balls, -15.0)], axis=1)
        speed = rng.uniform(20.0, 40.0, balls)
        yaw = np.radians(rng.uniform(-5.0, 5.0, balls))
        pitch = np.radians(rng.uniform(-5.0, 5.0, balls))
        vel = np.stack([np.sin(yaw) * np.cos(pitch), np.sin(pitch), np.cos(yaw) * np.cos(pitch)], axis=1) * speed[:, None]
        bb["position"][:, :3] = start.astype(np.float32)
        bb["velocity"][:, :3] = vel.astype(np.float32)
        cb = collider_descs(balls, np.arange(balls), abi.SHAPE_BALL, (0.4, 0, 0), density=10.0, friction=0.6)
        cb["ccd_enabled"] = 1 if ccd else 0
        parts_b += [g, b, bb]
        parts_c += [gc, c, cb]
    bodies, colliders = _concat(parts_b, parts_c)
    return Scene(f"{n_walls} brick walls", bodies, colliders, dt=1.0 / 120.0, steps=2000,
                 info={"walls": n_walls, "bodies": n_walls * (width * height + balls)})


# ---------------------------------------------------------------- compounds
def _qmul(a, b):
    """Quaternion product a * b, (i, j, k, w) order, float32."""
    ai, aj, ak, aw = a
    bi, bj, bk, bw = b
    return np.array([aw * bi + ai * bw + aj * bk - ak * bj, aw * bj - ai * bk + aj * bw + ak * bi,
                     aw * bk + ai * bj - aj * bi + ak * bw, aw * bw - ai * bi - aj * bj - ak * bk], np.float32)


def _qrot(q, v):
    i, j, k, w = q
    u = np.array([i, j, k], np.float32)
    t = 2.0 * np.cross(u, v)
    return (v + w * t + np.cross(u, t)).astype(np.float32)


def shape_mass_properties(shape, params, density):
    """(mass, centre, angular inertia about the centre) of a ball, cuboid or
    capsule in f64: volumetric_ball.rs, volumetric_cuboid.rs and
    volumetric_capsule.rs (the capsule's axis along local y)."""
    if shape == abi.SHAPE_BALL:
        r = float(params[0])
        m = density * 4.0 / 3.0 * np.pi * r ** 3
        return m, np.zeros(3), np.eye(3) * (m * 0.4 * r * r)
    if shape == abi.SHAPE_CUBOID:
        hx, hy, hz = (float(v) for v in params)
        m = density * 8.0 * hx * hy * hz
        return m, np.zeros(3), np.diag([hy * hy + hz * hz, hx * hx + hz * hz, hx * hx + hy * hy]) * (m / 3.0)
    r, hh = float(params[0]), float(params[1])
    m = density * (np.pi * r * r * 2.0 * hh + 4.0 / 3.0 * np.pi * r ** 3)
    h = 2.0 * hh
    unit = np.diag([(3.0 * r * r + h * h) / 12.0, r * r / 2.0, (3.0 * r * r + h * h) / 12.0]) + np.eye(3) * 0.4 * r * r
    extra = h * h * 0.5 + h * r * 3.0 / 8.0
    unit[0, 0] += extra
    unit[2, 2] += extra
    return m, np.zeros(3), unit * m


def _rotm(q):
    i, j, k, w = (float(v) for v in q)
    return np.array([[1 - 2 * (j * j + k * k), 2 * (i * j - k * w), 2 * (i * k + j * w)],
                     [2 * (i * j + k * w), 1 - 2 * (i * i + k * k), 2 * (j * k - i * w)],
                     [2 * (i * k - j * w), 2 * (j * k + i * w), 1 - 2 * (i * i + j * j)]])


def compound_mass_properties(parts, density):
    """Compound::mass_properties (volumetric_compound.rs): the parts' masses
    summed, their centres averaged by mass, their inertias rotated into the
    compound's frame, moved to the common centre and summed; in f64."""
    props = [(np.asarray(t, np.float64), _rotm(q)) + shape_mass_properties(sh, pr, 1.0) for t, q, sh, pr in parts]
    mt = sum(p[2] for p in props)
    com = sum((R @ c + t) * m for t, R, m, c, _ in props) / mt
    I = np.zeros((3, 3))
    for t, R, m, c, Ip in props:
        d = R @ c + t - com
        I += R @ Ip @ R.T + m * (np.dot(d, d) * np.eye(3) - np.outer(d, d))
    return mt * density, com, I * density


def add_collider_mass(body, mass, com, inertia):
    """RigidBody::add_local_inertia_and_com (rigid_body.rs:747-766) on a body
    description: the centre becomes the mass-weighted average, the inertias
    add (about their own centres, as the reference adds them)."""
    m0 = float(body["local_inertia"][0])
    c0 = np.asarray(body["local_com"], np.float64)
    ms = m0 + mass
    body["local_com"] = (c0 * m0 + np.asarray(com) * mass) / ms if ms != 0.0 else 0.0
    li = body["local_inertia"]
    li[0] = ms
    for k, (a, b) in enumerate(((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))):
        li[1 + k] += inertia[a, b]


def compound_colliders(body_index, parts, position=((0.0, 0.0, 0.0), (0.0, 0.0, 0.0, 1.0)), density=0.0,
                       friction=0.5, restitution=0.0):
    """ColliderDesc::new(ShapeHandle::new(Compound::new(parts))) on a body
    (ncollide3d's Compound): one collider per part, at the compound
    collider's position times the part's, sharing its material; each part
    collides on its own. The parts carry no density: the compound's mass
    properties (compound_mass_properties at `density`, moved by `position`
    as Volumetric::transformed_mass_properties does) are returned for
    add_collider_mass, which adds them to the body as the reference adds a
    collider's. `parts`: (translation, quaternion (i, j, k, w), shape,
    shape_params) per part. Returns (colliders, (mass, centre, inertia))."""
    t0 = np.asarray(position[0], np.float32)
    q0 = np.asarray(position[1], np.float32)
    out = []
    for t, q, shape, params in parts:
        c = collider_descs(1, body_index, shape, params, density=0.0, friction=friction, restitution=restitution)
        c["position_wrt_body"][0, :3] = t0 + _qrot(q0, np.asarray(t, np.float32))
        c["position_wrt_body"][0, 3:] = _qmul(q0, np.asarray(q, np.float32))
        out.append(c)
    m, com, I = compound_mass_properties(parts, density)
    R0 = _rotm(q0)
    return np.concatenate(out), (m, R0 @ com + t0.astype(np.float64), R0 @ I @ R0.T)


def compound_drop(n=6, seed=17, world=0):
    """Compound bodies dropped on the ground: L shapes of two cuboids,
    dumbbells of two balls on a capsule bar, and T shapes of a cuboid and a
    capsule, each with a random orientation."""
    rng = np.random.default_rng(seed)
    g, gc = _ground(half=(20.0, 1.0, 20.0), world=world)
    b = body_descs(n)
    b["world"] = world
    b["position"][:, 0] = (np.arange(n) % 3 - 1) * 3.0
    b["position"][:, 1] = 2.0 + 1.5 * (np.arange(n) // 3)
    b["position"][:, 3:] = uniform_quaternions(rng, n)
    qz = np.array([0.0, 0.0, np.sin(np.pi / 4), np.cos(np.pi / 4)], np.float32)   # local y onto x
    ident = (0.0, 0.0, 0.0, 1.0)
    kinds = [
        [((0.0, 0.0, 0.0), ident, abi.SHAPE_CUBOID, (0.6, 0.15, 0.2)),
         ((0.45, 0.45, 0.0), ident, abi.SHAPE_CUBOID, (0.15, 0.3, 0.2))],
        [((-0.6, 0.0, 0.0), ident, abi.SHAPE_BALL, (0.3, 0.0, 0.0)),
         ((0.6, 0.0, 0.0), ident, abi.SHAPE_BALL, (0.3, 0.0, 0.0)),
         ((0.0, 0.0, 0.0), qz, abi.SHAPE_CAPSULE, (0.08, 0.5, 0.0))],
        [((0.0, 0.3, 0.0), ident, abi.SHAPE_CUBOID, (0.5, 0.1, 0.1)),
         ((0.0, -0.2, 0.0), ident, abi.SHAPE_CAPSULE, (0.1, 0.3, 0.0))],
    ]
    cs = []
    for i in range(n):
        c, mp = compound_colliders(i, kinds[i % 3], density=1.0)
        add_collider_mass(b[i], *mp)
        cs.append(c)
    bodies, colliders = _concat([g, b], [gc, np.concatenate(cs)])
    return Scene("compound drop", bodies, colliders)


# ---------------------------------------------------------------- sensors
def sensor_gates(balls=6, sensors=True, seed=11, world=0):
    """Balls dropped through a static sensor box (a trigger zone above the
    ground) onto the ground; the first ball also carries a massless sensor
    ball of radius 0.9 around it (a proximity trigger moving with it). With
    `sensors` False the two sensor colliders are left out: the bodies' motion
    is the same, since sensors make no contacts and add no mass."""
    rng = np.random.default_rng(seed)
    g, gc = _ground(half=(10.0, 0.5, 10.0), world=world)
    zone = collider_descs(1, 0, abi.SHAPE_CUBOID, (1.5, 0.4, 1.5))
    zone["position_wrt_body"][0, 1] = 2.0
    zone["is_sensor"] = 1
    b = body_descs(balls)
    b["world"] = world
    b["position"][:, 0] = rng.uniform(-1.2, 1.2, balls).astype(np.float32)
    b["position"][:, 1] = (4.0 + 0.9 * np.arange(balls)).astype(np.float32)
    b["position"][:, 2] = rng.uniform(-1.2, 1.2, balls).astype(np.float32)
    c = collider_descs(balls, np.arange(balls), abi.SHAPE_BALL, (0.25, 0.0, 0.0), density=1.0, friction=0.5)
    trig = collider_descs(1, 0, abi.SHAPE_BALL, (0.9, 0.0, 0.0))
    trig["is_sensor"] = 1
    if sensors:
        bodies, colliders = _concat([g, b], [np.concatenate([gc, zone]), np.concatenate([c, trig])])
    else:
        bodies, colliders = _concat([g, b], [gc, c])
    return Scene("sensor gates", bodies, colliders)


# ---------------------------------------------------------------- CCD scenes
def ccd_wall(speed=120.0, half_thickness=0.05, radius=0.1, n=1, ccd=True, gravity=(0.0, 0.0, 0.0),
             shape=abi.SHAPE_BALL, spin=0.0, seed=3, world=0, restitution=0.0, linear_interp=False):
    """Fast projectiles at a thin static wall (a cuboid of half thickness
    `half_thickness` centred on the plane x = 0): at `speed` a projectile moves
    speed / 60 m a step, far more than the wall is thick, so it passes through
    it unless its collider has CCD enabled. Balls of `radius` (or cubes of
    that half extent, spun about z at `spin` rad/s) start at x = -1."""
    rng = np.random.default_rng(seed)
    g = ground_descs(1)
    g["world"] = world
    gc = collider_descs(1, 0, abi.SHAPE_CUBOID, (half_thickness, 2.0, 2.0), friction=0.5, restitution=restitution)
    gc["position_wrt_body"][0, 1] = 2.0
    b = body_descs(n)
    b["world"] = world
    b["position"][:, 0] = -1.0
    b["position"][:, 1] = rng.uniform(0.6, 3.4, n).astype(np.float32)
    b["position"][:, 2] = rng.uniform(-1.4, 1.4, n).astype(np.float32)
    b["velocity"][:, 0] = speed
    b["velocity"][:, 5] = spin
    if linear_interp:
        b["flags"] |= abi.BODY_LINEAR_INTERP
    params = (radius, 0.0, 0.0) if shape == abi.SHAPE_BALL else (radius, radius, radius)
    c = collider_descs(n, np.arange(n), shape, params, density=1.0, friction=0.5, restitution=restitution)
    c["ccd_enabled"] = 1 if ccd else 0
    bodies, colliders = _concat([g, b], [gc, c])
    return Scene("ccd wall", bodies, colliders, gravity=gravity)


def ccd_stack(height=4, speed=80.0, balls=3, ccd=True, seed=5, world=0):
    """A tower of `height` unit boxes on the ground struck by `balls` fast
    CCD balls (radius 0.2, 10 kg/m^3) flying at it along x: each impact's
    substep takes the struck box and, through their contacts, the boxes and
    balls touching it."""
    rng = np.random.default_rng(seed)
    g, gc = _ground(half=(20.0, 1.0, 20.0), world=world)
    b = body_descs(height)
    b["world"] = world
    b["position"][:, 1] = 0.5 + np.arange(height) * 1.0
    c = collider_descs(height, np.arange(height), abi.SHAPE_CUBOID, (0.5, 0.5, 0.5), density=1.0, friction=0.5)
    bb = body_descs(balls)
    bb["world"] = world
    bb["position"][:, 0] = -3.0
    bb["position"][:, 1] = (0.5 + rng.integers(0, height, balls) * 1.0 + rng.uniform(-0.3, 0.3, balls)).astype(np.float32)
    bb["position"][:, 2] = rng.uniform(-0.3, 0.3, balls).astype(np.float32)
    bb["velocity"][:, 0] = speed
    cb = collider_descs(balls, np.arange(balls), abi.SHAPE_BALL, (0.2, 0.0, 0.0), density=10.0, friction=0.5)
    cb["ccd_enabled"] = 1 if ccd else 0
    bodies, colliders = _concat([g, b, bb], [gc, c, cb])
    return Scene("ccd stack", bodies, colliders)


def batched_ccd(n_worlds=6, seed=7, worlds=None):
    """Worlds alternating a tower struck by CCD balls and fast CCD
    projectiles at a thin wall (balls and spinning cubes), under gravity;
    `worlds` builds only those."""
    worlds = range(n_worlds) if worlds is None else worlds
    parts = []
    for w in worlds:
        if w % 3 == 0:
            parts.append(ccd_stack(height=3 + w % 2, speed=60.0 + 5.0 * w, balls=2, seed=seed + w))
        else:
            sc = ccd_wall(n=3, shape=abi.SHAPE_BALL if w % 3 == 1 else abi.SHAPE_CUBOID, spin=10.0 * (w % 3),
                          speed=90.0 + 4.0 * w, seed=seed + w, gravity=(0.0, -9.81, 0.0))
            parts.append(sc)
    return concat_worlds(parts, f"{len(parts)} CCD worlds")


# ---------------------------------------------------------------- small scenes
def single_body(shape=abi.SHAPE_CUBOID, params=(0.5, 0.5, 0.5), position=(0, 5, 0), velocity=(0, 0, 0, 0, 0, 0),
                rotation=(0, 0, 0, 1), ground=True, density=1.0, friction=0.5, restitution=0.0):
    parts_b, parts_c = [], []
    if ground:
        g, gc = _ground(friction=friction)
        parts_b.append(g)
        parts_c.append(gc)
    b = body_descs(1)
    b["position"][0, :3] = position
    b["position"][0, 3:7] = rotation
    b["velocity"][0] = velocity
    c = collider_descs(1, 0, shape, params, density=density, friction=friction, restitution=restitution)
    parts_b.append(b)
    parts_c.append(c)
    bodies, colliders = _concat(parts_b, parts_c)
    return Scene("single body", bodies, colliders)


def random_cluster(n=64, seed=7, extent=3.0, boxes=True, balls=True, ground=True, rotate=True, world=0,
                   capsules=False):
    """A small random cluster of balls and cuboids (and, with capsules=True,
    every third body a capsule of radius U(0.15, 0.5) and half height
    U(0.2, 0.8)) with overlaps, for collision-detection and solver parity
    checks."""
    rng = np.random.default_rng(seed)
    parts_b, parts_c = [], []
    if ground:
        g, gc = _ground(world=world)
        parts_b.append(g)
        parts_c.append(gc)
    b = body_descs(n)
    b["world"] = world
    b["position"][:, 0] = rng.uniform(-extent, extent, n)
    b["position"][:, 1] = rng.uniform(0.2, 2 * extent, n)
    b["position"][:, 2] = rng.uniform(-extent, extent, n)
    if rotate:
        b["position"][:, 3:7] = uniform_quaternions(rng, n)
    b["velocity"][:, :3] = rng.uniform(-1, 1, (n, 3))
    b["velocity"][:, 3:] = rng.uniform(-1, 1, (n, 3))
    kinds = rng.random(n)
    if boxes and not balls:
        is_ball = np.zeros(n, bool)
    elif balls and not boxes:
        is_ball = np.ones(n, bool)
    else:
        is_ball = kinds < 0.5
    c = collider_descs(n, np.arange(n), abi.SHAPE_BALL, (0, 0, 0), density=1.0, friction=0.5)
    c["shape"] = np.where(is_ball, abi.SHAPE_BALL, abi.SHAPE_CUBOID)
    p = np.zeros((n, 3), np.float32)
    p[is_ball, 0] = rng.uniform(0.2, 0.8, int(is_ball.sum()))
    p[~is_ball] = rng.uniform(0.2, 0.8, (int((~is_ball).sum()), 3))
    c["shape_params"] = p
    if capsules:
        cap = np.arange(n) % 3 == 2
        c["shape"][cap] = abi.SHAPE_CAPSULE
        c["shape_params"][cap] = np.stack([rng.uniform(0.15, 0.5, int(cap.sum())),
                                           rng.uniform(0.2, 0.8, int(cap.sum())),
                                           np.zeros(int(cap.sum()))], axis=1)
    parts_b.append(b)
    parts_c.append(c)
    bodies, colliders = _concat(parts_b, parts_c)
    return Scene(f"random cluster ({n})", bodies, colliders)


def _qmul(a, b):
    """Hamilton product of (i, j, k, w) quaternions (float64)."""
    ai, aj, ak, aw = a
    bi, bj, bk, bw = b
    return np.array([aw * bi + ai * bw + aj * bk - ak * bj, aw * bj - ai * bk + aj * bw + ak * bi,
                     aw * bk + ai * bj - aj * bi + ak * bw, aw * bw - ai * bi - aj * bj - ak * bk])


def _qconj(q):
    return np.array([-q[0], -q[1], -q[2], q[3]])


def _qrot(q, v):
    u, w = np.asarray(q[:3], np.float64), float(q[3])
    t = 2.0 * np.cross(u, v)
    return np.asarray(v, np.float64) + w * t + np.cross(u, t)


def _jointed_world(rng, world, chains, links, clusters, balls, ground_half=(20.0, 1.0, 20.0)):
    """One world of jointed bodies on its own ground (body 0 of the world):
    `chains` chains of `links` cuboids joined end to end by ball joints, the
    first hanging from a pivot on the ground body, laid out horizontally so
    they swing down onto the ground; `clusters` pairs of a cuboid and a ball
    held by a fixed joint at their midpoint (random reference frames chosen
    so the start satisfies the joint), thrown tumbling onto the ground; and
    `balls` free balls. Adjacent links keep a gap so their boxes do not touch."""
    g, gc = _ground(half=ground_half, world=world)
    bodies, colliders, joints = [g], [gc], []
    nb = 1
    hl, gap = 0.25, 0.05                  # link half length, gap at each joint
    for c in range(chains):
        pivot = np.array([rng.uniform(-6, 6), rng.uniform(3.0, 5.0), rng.uniform(-6, 6)])
        yaw = rng.uniform(0, 2 * np.pi)
        axis = np.array([np.cos(yaw), 0.0, np.sin(yaw)])
        q = np.array([0.0, np.sin(-yaw / 2), 0.0, np.cos(-yaw / 2)])   # local x -> axis
        b = body_descs(links)
        b["world"] = world
        for i in range(links):
            centre = pivot + axis * (gap + hl + i * (2 * hl + 2 * gap))
            b["position"][i, :3] = centre
            b["position"][i, 3:7] = q
        cl = collider_descs(links, np.arange(links) + nb, abi.SHAPE_CUBOID, (hl, 0.08, 0.08), density=2.0,
                            friction=0.4)
        bodies.append(b)
        colliders.append(cl)
        j = joint_descs(links)
        j["kind"] = abi.JOINT_BALL
        for i in range(links):
            if i == 0:
                j["body1"]["index"][i] = 0
                j["anchor1"][i] = pivot
            else:
                j["body1"]["index"][i] = nb + i - 1
                j["anchor1"][i] = (hl + gap, 0.0, 0.0)
            j["body2"]["index"][i] = nb + i
            j["anchor2"][i] = (-(hl + gap), 0.0, 0.0)
        joints.append(j)
        nb += links
    for c in range(clusters):
        t1 = np.array([rng.uniform(-6, 6), rng.uniform(2.0, 6.0), rng.uniform(-6, 6)])
        q1 = uniform_quaternions(rng, 1)[0].astype(np.float64)
        off = _qrot(q1, np.array([0.0, 0.0, 0.75]))
        t2 = t1 + off
        q2 = uniform_quaternions(rng, 1)[0].astype(np.float64)
        b = body_descs(2)
        b["world"] = world
        b["position"][0, :3], b["position"][0, 3:7] = t1, q1
        b["position"][1, :3], b["position"][1, 3:7] = t2, q2
        v = rng.uniform(-2, 2, 6)
        b["velocity"][:] = v
        cl = collider_descs(2, np.arange(2) + nb, abi.SHAPE_CUBOID, (0.3, 0.2, 0.25), density=1.0, friction=0.5)
        cl["shape"][1] = abi.SHAPE_BALL
        cl["shape_params"][1] = (0.3, 0.0, 0.0)
        bodies.append(b)
        colliders.append(cl)
        mid = (t1 + t2) / 2
        f1 = uniform_quaternions(rng, 1)[0].astype(np.float64)
        f2 = _qmul(_qmul(_qconj(q2), q1), f1)           # q2 f2 = q1 f1 at the start
        j = joint_descs(1)
        j["kind"] = abi.JOINT_FIXED
        j["body1"]["index"][0], j["body2"]["index"][0] = nb, nb + 1
        j["anchor1"][0] = _qrot(_qconj(q1), mid - t1)
        j["anchor2"][0] = _qrot(_qconj(q2), mid - t2)
        j["frame1"][0], j["frame2"][0] = f1, f2 / np.linalg.norm(f2)
        joints.append(j)
        nb += 2
    if balls:
        b = body_descs(balls)
        b["world"] = world
        b["position"][:, 0] = rng.uniform(-6, 6, balls)
        b["position"][:, 1] = rng.uniform(1.0, 6.0, balls)
        b["position"][:, 2] = rng.uniform(-6, 6, balls)
        b["velocity"][:, :3] = rng.uniform(-3, 3, (balls, 3))
        cl = collider_descs(balls, np.arange(balls) + nb, abi.SHAPE_BALL, (0.3, 0, 0), density=1.0, friction=0.5)
        bodies.append(b)
        colliders.append(cl)
        nb += balls
    return np.concatenate(bodies), np.concatenate(colliders), np.concatenate(joints), nb


def jointed(chains=4, links=8, clusters=6, balls=10, seed=3):
    """Ball-jointed chains swinging from pivots on the ground body, fixed-jointed
    cuboid-ball pairs and free balls, falling onto the ground: the joint
    parity scene (one world)."""
    rng = np.random.default_rng(seed)
    bodies, colliders, joints, _ = _jointed_world(rng, 0, chains, links, clusters, balls)
    sc = Scene("jointed bodies", bodies, colliders, steps=120)
    return set_joints(sc, joints)


def batched_jointed(n_worlds=8, seed=5, chains=2, links=6, clusters=3, balls=4, worlds=None):
    """Independent worlds of the jointed scene, each on its own ground (joint
    and body slots renumbered per world in order): the per-world schedule
    with joints. `worlds` builds only those worlds, renumbered from world 0."""
    worlds = range(n_worlds) if worlds is None else worlds
    parts_b, parts_c, parts_j = [], [], []
    off = 0
    for local, w in enumerate(worlds):
        rng = np.random.default_rng([seed, w])
        b, c, j, nb = _jointed_world(rng, local, chains, links, clusters, balls)
        c = c.copy()
        c["body"]["index"] += off
        j = j.copy()
        j["body1"]["index"] += off
        j["body2"]["index"] += off
        parts_b.append(b)
        parts_c.append(c)
        parts_j.append(j)
        off += nb
    sc = Scene(f"{len(worlds)} jointed worlds", np.concatenate(parts_b), np.concatenate(parts_c), steps=120)
    return set_joints(sc, np.concatenate(parts_j))


def pendulum(length=2.0, angle=0.2, radius=0.1, density=100.0, chain=1):
    """A ball on a massless rod: a ball joint between a pivot on the ground
    body (at height 10) and the ball, `length` below it, released at `angle`
    from the vertical; with chain > 1 the balls hang one below the other.
    No collisions occur (the balls stay far from the ground)."""
    g = ground_descs(1)
    gc = collider_descs(1, 0, abi.SHAPE_CUBOID, (1.0, 1.0, 1.0))
    gc["position_wrt_body"][0, 1] = -1.0
    b = body_descs(chain)
    pivot = np.array([0.0, 10.0, 0.0])
    d = np.array([np.sin(angle), -np.cos(angle), 0.0])
    for i in range(chain):
        b["position"][i, :3] = pivot + d * length * (i + 1)
    b["flags"] = abi.BODY_GRAVITY          # never sleeps
    c = collider_descs(chain, np.arange(chain), abi.SHAPE_BALL, (radius, 0, 0), density=density)
    bodies, colliders = _concat([g, b], [gc, c])
    j = joint_descs(chain)
    j["kind"] = abi.JOINT_BALL
    for i in range(chain):
        j["body1"]["index"][i] = i          # the ground, then the ball above
        j["anchor1"][i] = pivot if i == 0 else (0.0, 0.0, 0.0)
        j["body2"]["index"][i] = i + 1
        j["anchor2"][i] = -d * length if i == 0 else -d * length
    sc = Scene("pendulum", bodies, colliders, steps=600)
    return set_joints(sc, j)


def hinge(kind=abi.JOINT_REVOLUTE, half=(0.5, 0.1, 0.1), angle=0.3, density=1.0, spin=(0.0, 0.0, 0.0)):
    """A box hung from the ground body (the pivot at height 10) by one joint of
    `kind`: its -x end at the pivot, the body tilted by `angle` about z from
    the horizontal +x direction; the joint axes are z in both frames
    (revolute: a physical pendulum swinging in the x-y plane), and the box
    starts with angular velocity `spin`. No collisions occur."""
    g = ground_descs(1)
    gc = collider_descs(1, 0, abi.SHAPE_CUBOID, (1.0, 1.0, 1.0))
    gc["position_wrt_body"][0, 1] = -1.0
    b = body_descs(1)
    pivot = np.array([0.0, 10.0, 0.0])
    c, s_ = math.cos(-angle), math.sin(-angle)
    b["position"][0, :3] = pivot + np.array([c, s_, 0.0]) * half[0]
    b["position"][0, 3:7] = (0.0, 0.0, math.sin(-angle / 2), math.cos(-angle / 2))
    b["velocity"][0, 3:] = spin
    b["flags"] = abi.BODY_GRAVITY
    cl = collider_descs(1, 0, abi.SHAPE_CUBOID, half, density=density)
    bodies, colliders = _concat([g, b], [gc, cl])
    j = joint_descs(1)
    j["kind"] = kind
    j["body1"]["index"], j["body2"]["index"] = 0, 1
    j["anchor1"][0] = pivot
    j["anchor2"][0] = (-half[0], 0.0, 0.0)
    q = np.array([0.0, 0.0, math.sin(-angle / 2), math.cos(-angle / 2)])
    j["frame1"][0] = q                        # frames equal at the start: ground frame = body rotation
    j["frame2"][0] = (0.0, 0.0, 0.0, 1.0)
    j["axis1"][0] = (0.0, 0.0, 1.0)
    j["axis2"][0] = (0.0, 0.0, 1.0)
    sc = Scene("hinge", bodies, colliders, steps=600)
    return set_joints(sc, j)


def joint_zoo(seed=11, world=0, ground=True):
    """One of each joint kind on boxes and balls over the ground, with
    random initial velocities, plus a few free boxes falling on them: the
    joint-kind parity scene. Revolute, universal and fixed pairs join two
    dynamic bodies; cartesian, planar and rectangular joints hold a body to
    the ground body."""
    rng = np.random.default_rng(seed)
    parts_b, parts_c, joints = [], [], []
    g, gc = _ground(half=(20.0, 1.0, 20.0), world=world)
    parts_b.append(g)
    parts_c.append(gc)
    nb = 1
    kinds = [abi.JOINT_BALL, abi.JOINT_FIXED, abi.JOINT_REVOLUTE, abi.JOINT_CARTESIAN, abi.JOINT_PLANAR,
             abi.JOINT_RECTANGULAR, abi.JOINT_UNIVERSAL, abi.JOINT_PRISMATIC, abi.JOINT_CYLINDRICAL, abi.JOINT_PIN_SLOT]
    for i, kind in enumerate(kinds):
        x = -13.5 + 3.0 * i
        two = kind in (abi.JOINT_BALL, abi.JOINT_FIXED, abi.JOINT_REVOLUTE, abi.JOINT_UNIVERSAL,
                       abi.JOINT_CYLINDRICAL, abi.JOINT_PIN_SLOT)
        n = 2 if two else 1
        b = body_descs(n)
        b["world"] = world
        b["position"][0, :3] = (x, 2.5, 0.0)
        if two:
            b["position"][1, :3] = (x + 0.8, 2.5, 0.0)
        b["velocity"][:] = rng.uniform(-1.5, 1.5, (n, 6))
        cl = collider_descs(n, np.arange(n), abi.SHAPE_CUBOID, (0.3, 0.2, 0.25), density=1.0, friction=0.5)
        if two:
            cl["shape"][1] = abi.SHAPE_BALL
            cl["shape_params"][1] = (0.25, 0.0, 0.0)
        parts_b.append(b)
        parts_c.append(cl)
        j = joint_descs(1)
        j["kind"] = kind
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        if two:
            j["body1"]["index"], j["body2"]["index"] = nb, nb + 1
            j["anchor1"][0] = (0.4, 0.0, 0.0)
            j["anchor2"][0] = (-0.4, 0.0, 0.0)
            perp = np.cross(ax, (0.0, 1.0, 0.0)) / np.linalg.norm(np.cross(ax, (0.0, 1.0, 0.0)))
            j["axis1"][0] = ax
            j["axis2"][0] = ax if kind != abi.JOINT_UNIVERSAL else perp
            if kind == abi.JOINT_UNIVERSAL:
                j["angle"][0] = math.pi / 2
            if kind == abi.JOINT_PIN_SLOT:
                j["axis1"][0] = (1.0, 0.0, 0.0)      # the slot (axis_v1)
                j["axis3"][0] = perp                 # the pin's axis on body 1 (axis_w1) ...
                j["axis2"][0] = perp                 # ... and on body 2 (axis_w2)
        else:
            j["body1"]["index"], j["body2"]["index"] = 0, nb
            j["anchor1"][0] = (x, 2.5, 0.0)
            j["anchor2"][0] = (0.0, 0.0, 0.0)
            j["axis1"][0] = (0.0, 1.0, 0.0) if kind != abi.JOINT_RECTANGULAR else ax
            j["axis2"][0] = (0.0, 1.0, 0.0)
            if kind == abi.JOINT_PRISMATIC:
                # A vertical slider that falls onto its lower offset limit.
                j["limit_flags"][0] = abi.JOINT_MIN_OFFSET | abi.JOINT_MAX_OFFSET
                j["min_offset"][0], j["max_offset"][0] = -1.0, 0.5
        joints.append(j)
        nb += n
    drops = body_descs(6)
    drops["world"] = world
    drops["position"][:, 0] = -13.5 + 3.0 * rng.integers(0, len(kinds), 6) + rng.uniform(-0.3, 0.3, 6)
    drops["position"][:, 1] = rng.uniform(4.0, 7.0, 6)
    drops["position"][:, 2] = rng.uniform(-0.3, 0.3, 6)
    drops["position"][:, 3:7] = uniform_quaternions(rng, 6)
    dc = collider_descs(6, np.arange(6), abi.SHAPE_CUBOID, (0.2, 0.2, 0.2), density=1.0, friction=0.5)
    parts_b.append(drops)
    parts_c.append(dc)
    bodies, colliders = _concat(parts_b, parts_c)
    sc = Scene("joint zoo", bodies, colliders, steps=240)
    return set_joints(sc, np.concatenate(joints))


def concat_worlds(parts, name="batched worlds"):
    """Scenes of one world each, side by side as the worlds 0, 1, ... of one
    batch: body slots follow each other, collider parents and joint bodies are
    renumbered, and each scene's bodies take its world index."""
    bodies, colliders, joints = [], [], []
    off = 0
    for wd, sc in enumerate(parts):
        b = sc.bodies.copy()
        b["world"] = wd
        c = sc.colliders.copy()
        c["body"]["index"] += off
        j = sc.joints.copy()
        j["body1"]["index"] += off
        j["body2"]["index"] += off
        bodies.append(b)
        colliders.append(c)
        joints.append(j)
        off += len(b)
    sc = Scene(name, np.concatenate(bodies), np.concatenate(colliders), gravity=parts[0].gravity, steps=parts[0].steps)
    return set_joints(sc, np.concatenate(joints))


def batched_zoo(n_worlds=6, seed=11, worlds=None):
    """Worlds of the joint zoo (seeds seed, seed + 1, ...); `worlds` builds only those."""
    worlds = range(n_worlds) if worlds is None else worlds
    return concat_worlds([joint_zoo(seed=seed + w) for w in worlds], f"{len(worlds)} joint-zoo worlds")

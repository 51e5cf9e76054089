"""Parity of the GPU step (through the C ABI) with the CPU oracle.

The GPU solver visits manifolds colour by colour; the oracle's colour order
(ORDER_COLOUR) is the same Gauss-Seidel sequence written sequentially, and
both evaluate every expression in the same order without fused multiply-add.
Tolerances: 1e-5 relative on contact geometry, 1e-4 relative on impulses,
1e-3 on 1000-step resting poses (the bars the path is specified to).
"""
import numpy as np
import pytest

from nphysics_gb300 import abi, scenes
from oracle.oracle_py import ORDER_COLOUR, ORDER_REFERENCE, OracleWorld

pytestmark = pytest.mark.gpu


def make_pair(scene, params=None, precision=32, order=ORDER_COLOUR, pairs_per_collider=16):
    from nphysics_gb300.world import GpuWorld
    p = params if params is not None else scene.params()
    g = GpuWorld.for_scene(scene, p, pairs_per_collider=pairs_per_collider)
    o = OracleWorld(p, scene.gravity, precision=precision, order=order)
    o.load_scene(scene)
    return g, o


def contact_table(c):
    key = (c["collider1"].astype(np.uint64) << np.uint64(40)) | (c["collider2"].astype(np.uint64) << np.uint64(10)) | \
        c["feature_key"].astype(np.uint64)
    order = np.argsort(key, kind="stable")
    return key[order], {k: v[order] for k, v in c.items()}


def assert_close_rel(a, b, rtol, atol, what):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    err = np.abs(a - b)
    bound = atol + rtol * np.abs(b)
    bad = err > bound
    assert not bad.any(), f"{what}: {bad.sum()} of {bad.size} beyond tolerance; max err {err.max():.3e}"


def test_mass_properties_match(gpu_lib):
    sc = scenes.random_cluster(n=40, seed=11)
    g, o = make_pair(sc)
    g.step(1)
    o.step(1)
    gi, gc = g.mass_properties()
    oi, oc = o.mass_properties()
    assert_close_rel(gi, oi, 1e-6, 1e-7, "local inertia")
    assert_close_rel(gc, oc, 1e-6, 1e-7, "local com")


def test_free_motion_no_contacts(gpu_lib):
    # Spinning, falling bodies far apart: update_dynamics (gyroscopic augmented
    # mass), update_acceleration and integrate only.
    sc = scenes.random_cluster(n=32, seed=5, extent=400.0, ground=False)
    sc.bodies["velocity"][:, 3:] *= 5.0
    g, o = make_pair(sc)
    for _ in range(3):
        g.step(10)
        o.step(10)
        gb, ob = g.bodies(), o.bodies()
        assert_close_rel(gb["position"], ob["position"], 1e-6, 1e-6, "positions")
        assert_close_rel(gb["velocity"], ob["velocity"], 1e-6, 1e-6, "velocities")
    assert g.counters()["num_contacts"] == 0


def test_broad_phase_is_the_brute_force_set(gpu_lib):
    sc = scenes.random_cluster(n=400, seed=9, extent=5.0)
    g, o = make_pair(sc)
    g.step(2)
    pairs = g.pairs()
    aabb = g.aabbs()
    body = sc.colliders["body"]["index"].astype(np.int64)
    status = sc.bodies["status"]
    n = len(aabb)
    mn, mx = aabb[:, :3], aabb[:, 3:]
    ov = np.all((mn[:, None, :] <= mx[None, :, :]) & (mn[None, :, :] <= mx[:, None, :]), axis=2)
    iu = np.triu_indices(n, 1)
    ok = ov[iu] & (body[iu[0]] != body[iu[1]]) & ((status[body[iu[0]]] == abi.BODY_DYNAMIC) |
                                                  (status[body[iu[1]]] == abi.BODY_DYNAMIC))
    brute = np.stack([iu[0][ok], iu[1][ok]], axis=1).astype(np.uint32)
    assert len(pairs) > 200
    np.testing.assert_array_equal(pairs, brute)


def test_broad_phase_and_aabbs_match_oracle(gpu_lib):
    sc = scenes.random_cluster(n=200, seed=2, extent=4.0)
    g, o = make_pair(sc)
    g.step(1)
    o.step(1)
    np.testing.assert_array_equal(g.pairs(), o.pairs())
    assert_close_rel(g.aabbs(), o.aabbs(), 1e-6, 1e-6, "fat AABBs")


@pytest.mark.parametrize("boxes,balls", [(True, False), (False, True), (True, True)])
def test_contacts_match_oracle(gpu_lib, boxes, balls):
    sc = scenes.random_cluster(n=120, seed=17, extent=2.5, boxes=boxes, balls=balls)
    g, o = make_pair(sc)
    g.step(1)
    o.step(1)
    kg, cg = contact_table(g.contacts())
    ko, co = contact_table(o.contacts())
    assert len(kg) > 50
    np.testing.assert_array_equal(kg, ko)
    for f in ("world1", "world2", "normal"):
        assert_close_rel(cg[f], co[f], 1e-5, 1e-5, f)
    assert_close_rel(cg["depth"], co["depth"], 1e-5, 1e-5, "depth")
    assert_close_rel(cg["impulse"], co["impulse"], 1e-4, 1e-6, "impulses")


def test_single_step_impulses_pyramid(gpu_lib):
    sc = scenes.pyramid(base=20)
    g, o = make_pair(sc)
    g.step(1)
    o.step(1)
    kg, cg = contact_table(g.contacts())
    ko, co = contact_table(o.contacts())
    np.testing.assert_array_equal(kg, ko)
    assert_close_rel(cg["impulse"], co["impulse"], 1e-4, 1e-6, "impulses")
    cgc, coc = g.counters(), o.counters()
    assert cgc["num_colours"] == coc["num_colours"]
    assert cgc["num_solver_contacts"] == coc["num_solver_contacts"]
    assert abs(cgc["residual"] - coc["residual"]) <= 1e-6 * max(1.0, coc["residual"])


def test_converged_velocities_match_reference_order(gpu_lib):
    # Run to a tight residual: the colour order and the reference's order reach
    # the same velocities.
    sc = scenes.pyramid(base=8)
    p = sc.params()
    p.solve_to_tolerance = 1
    p.residual_tolerance = 1e-6      # f32 state bottoms out near 1e-7
    p.max_iterations_to_tolerance = 4000
    p.max_position_iterations = 0
    g, o = make_pair(sc, params=p, precision=64, order=ORDER_REFERENCE)
    g.step(1)
    o.step(1)
    assert g.counters()["residual"] <= 1e-6
    assert_close_rel(g.bodies()["velocity"], o.bodies()["velocity"], 1e-4, 1e-5, "converged velocities")


@pytest.mark.parametrize("sched", [abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS])
def test_capsule_cluster_matches_oracle(gpu_lib, sched):
    # Balls, cuboids and capsules tumbling onto the ground: mass properties,
    # contacts and 150 steps of poses against the oracle in the colour order,
    # bit for bit.
    sc = scenes.random_cluster(n=90, seed=23, extent=2.5, capsules=True)
    p = sc.params()
    p.solver_schedule = sched
    g, o = make_pair(sc, params=p)
    g.step(1)
    o.step(1)
    gi, gcom = g.mass_properties()
    oi, ocom = o.mass_properties()
    assert_close_rel(gi, oi, 1e-6, 1e-7, "local inertia")
    kg, cg = contact_table(g.contacts())
    ko, co = contact_table(o.contacts())
    np.testing.assert_array_equal(kg, ko)
    assert len(kg) > 30
    for f in ("world1", "world2", "normal", "depth"):
        assert_close_rel(cg[f], co[f], 1e-5, 1e-5, f)
    g.step(149)
    o.step(149)
    np.testing.assert_array_equal(g.bodies()["position"], o.bodies()["position"])
    np.testing.assert_array_equal(g.bodies()["velocity"], o.bodies()["velocity"])
    np.testing.assert_array_equal(g.pairs(), o.pairs())


@pytest.mark.parametrize("sched", [abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS])
def test_manifold_sweep_order_matches_oracle(gpu_lib, sched):
    # NPGPU_SWEEP_MANIFOLD (each manifold's friction rows, then its normal
    # rows, one sweep per iteration) on the GPU equals the oracle's same order
    # bit for bit, with the learned start and without.
    from oracle import mlp_ref
    for sc in (scenes.random_cluster(n=80, seed=31, extent=2.5, capsules=True),
               scenes.batched_worlds(n_worlds=5, seed=4, lo=8, hi=60)):
        for mode in (abi.WARMSTART_CACHE, abi.WARMSTART_LEARNED_ALL):
            p = sc.params()
            p.solver_schedule = sched
            p.sweep_order = abi.SWEEP_MANIFOLD
            p.warmstart_mode = mode
            g, o = make_pair(sc, params=p)
            if mode == abi.WARMSTART_LEARNED_ALL:
                net = mlp_ref.random_params(np.random.default_rng(9))
                net[mlp_ref.YS:mlp_ref.PARAMS] = 0.05
                g.mlp_set(net)
                o.mlp_set(net)
            g.step(40)
            o.step(40)
            np.testing.assert_array_equal(g.bodies()["position"], o.bodies()["position"])
            np.testing.assert_array_equal(g.bodies()["velocity"], o.bodies()["velocity"])


def ball_stack(k, radius=0.5):
    """k balls stacked vertically, each touching the next, the lowest on the ground."""
    g, gc = scenes._ground(friction=0.5)
    b = scenes.body_descs(k)
    b["position"][:, 0] = 0.3
    b["position"][:, 1] = radius + 2 * radius * np.arange(k)
    b["position"][:, 2] = -0.7
    c = scenes.collider_descs(k, np.arange(k), abi.SHAPE_BALL, (radius, 0, 0), density=1.0, friction=0.5)
    bodies, colliders = scenes._concat([g, b], [gc, c])
    return scenes.Scene(f"stack of {k} balls", bodies, colliders)


@pytest.mark.parametrize("k", [1, 2, 5])
def test_converged_impulses_match_f64(gpu_lib, k):
    # A ball on the ground and stacks of balls: one contact per touching pair,
    # so the converged impulses are unique. A single step from rest solved to a
    # tight residual: the GPU (f32, colour order) matches the f64 oracle in the
    # reference's order within 1e-4 relative, and both match the statics:
    # contact i from the top carries i ball weights, m g dt each.
    from nphysics_gb300.world import GpuWorld
    sc = ball_stack(k)
    p = sc.params()
    p.solve_to_tolerance = 1
    p.residual_tolerance = 1e-6
    p.max_iterations_to_tolerance = 4000
    g = GpuWorld.for_scene(sc, p)
    g.step(1)
    q = sc.params()
    q.solve_to_tolerance = 1
    q.residual_tolerance = 1e-12
    q.max_iterations_to_tolerance = 4000
    o = OracleWorld(q, sc.gravity, precision=64, order=ORDER_REFERENCE)
    o.load_scene(sc)
    o.step(1)
    kg, cg = contact_table(g.contacts())
    oc = o.contacts()                      # keys, in the same order as the f64 rows
    oc["impulse"] = o.contacts_f64()[:, 10:13]
    ko, co = contact_table(oc)
    np.testing.assert_array_equal(kg, ko)
    assert len(kg) == k
    assert_close_rel(cg["impulse"][:, 0], co["impulse"][:, 0], 1e-4, 0.0, "converged normal impulses")
    m = 4.0 / 3.0 * np.pi * 0.5 ** 3
    # The contact with the ground is (0, 1); ball j sits on ball j - 1.
    weights = np.array([k - (int(c2) - 1) for c2 in cg["collider2"]], np.float64)
    assert_close_rel(cg["impulse"][:, 0], weights * m * 9.81 / 60.0, 1e-4, 0.0, "statics")
    assert np.abs(cg["impulse"][:, 1:]).max() <= 1e-6


def test_pyramid_1000_steps_resting_poses(gpu_lib):
    sc = scenes.pyramid(base=20)
    g, o = make_pair(sc)
    g.step(1000)
    o.step(1000)
    gp, op = g.bodies()["position"], o.bodies()["position"]
    assert np.abs(gp[:, :3] - op[:, :3]).max() < 1e-3
    assert np.abs(np.abs(gp[:, 3:]) - np.abs(op[:, 3:])).max() < 1e-3
    # Against the f64 oracle. The pyramid does not rest exactly: its layers
    # first separate by the collider margins (the top box rises 0.24-0.28 m),
    # and at 8 velocity iterations the stack creeps sideways at a rate that
    # depends on the Gauss-Seidel order and the precision. Measured drifts
    # after 1000 steps (maximum over boxes and axes):
    #   GPU (= f32 oracle, colour order) vs f64 oracle, colour order: 0.054 m
    #   GPU vs f64 oracle, the reference's order:                     0.328 m
    #   f64 colour order vs f64 reference order (the orders alone):   0.275 m
    #   f32 vs f64, both in the reference's order:                    0.027 m
    # The bounds are those measurements with a 20 % margin.
    def run(prec, order):
        w = OracleWorld(sc.params(), sc.gravity, precision=prec, order=order)
        w.load_scene(sc)
        w.step(1000)
        return w.bodies()["position"][:, :3]
    assert np.abs(gp[:, :3] - run(64, ORDER_COLOUR)).max() <= 0.065
    assert np.abs(gp[:, :3] - run(64, ORDER_REFERENCE)).max() <= 0.40
    assert g.counters()["max_penetration"] < 0.05
    assert g.bodies()["active"].sum() == 0   # the whole stack fell asleep, as in the oracle
    assert o.bodies()["active"].sum() == 0


def test_ball_pile_statistics(gpu_lib):
    sc = scenes.ball_pile(side=8)
    g, o = make_pair(sc)
    g.step(120)
    o.step(120)
    cg, co = g.counters(), o.counters()
    # Same Gauss-Seidel order: the chaotic pile agrees with the oracle.
    assert abs(cg["kinetic_energy"] - co["kinetic_energy"]) <= 1e-3 * max(co["kinetic_energy"], 1.0)
    assert abs(cg["max_penetration"] - co["max_penetration"]) <= 1e-4
    assert cg["num_contacts"] == co["num_contacts"]
    # Against the reference's order: stated bounds on energy, penetration and contacts.
    r = OracleWorld(sc.params(), sc.gravity, precision=32, order=ORDER_REFERENCE)
    r.load_scene(sc)
    r.step(120)
    cr = r.counters()
    assert abs(cg["kinetic_energy"] - cr["kinetic_energy"]) <= 0.05 * cr["kinetic_energy"]
    assert cg["max_penetration"] <= 1.5 * cr["max_penetration"] + 0.01
    assert abs(cg["num_contacts"] - cr["num_contacts"]) <= 0.05 * cr["num_contacts"]


def test_brick_walls_statistics_against_f64(gpu_lib):
    # Two of the brick-wall worlds (50 x 40 bricks, 64 balls at 20-40 m/s,
    # dt 1/120), 240 steps: the GPU equals the f32 oracle in the colour order
    # bit for bit; against the f64 oracle in the reference's order the
    # impacts are chaotic, so the bounds are on the statistics. Measured
    # (the GPU's run is the f32 oracle's): kinetic energy within 2.6 % of the
    # initial energy at every step, maximum penetration 0.314 m against
    # 0.320 m, 4911 against 4713 contacts at the end. The bounds below add
    # about 50 % to those gaps.
    sc = scenes.brick_walls(n_walls=2, width=50, height=40, balls=64, seed=1234)
    g, o = make_pair(sc, pairs_per_collider=8)
    r = OracleWorld(sc.params(), sc.gravity, precision=64, order=ORDER_REFERENCE)
    r.load_scene(sc)
    ke_g, ke_r, pen_g, pen_r = [], [], [], []
    for k in range(240):
        g.step(1)
        r.step(1)
        cg, cr = g.counters(), r.counters()
        ke_g.append(cg["kinetic_energy"])
        ke_r.append(cr["kinetic_energy"])
        pen_g.append(cg["max_penetration"])
        pen_r.append(cr["max_penetration"])
    o.step(240)
    np.testing.assert_array_equal(g.bodies()["position"], o.bodies()["position"])
    ke_g, ke_r = np.array(ke_g), np.array(ke_r)
    assert np.max(np.abs(ke_g - ke_r)) <= 0.04 * ke_r[0]
    assert abs(max(pen_g) - max(pen_r)) <= 0.02 + 0.05 * max(pen_r)
    assert abs(cg["num_contacts"] - cr["num_contacts"]) <= 0.08 * cr["num_contacts"]


def test_batched_worlds_do_not_interact(gpu_lib):
    # Two copies of a cluster in the same place but in different worlds: no
    # cross-world pair, and both follow the oracle. (A copy's slots differ, so
    # its colouring, hence its Gauss-Seidel order, differs from the original.)
    one = scenes.random_cluster(n=30, seed=4, world=0)
    two_b = np.concatenate([one.bodies, one.bodies.copy()])
    two_b["world"][len(one.bodies):] = 1
    two_c = np.concatenate([one.colliders, one.colliders.copy()])
    two_c["body"]["index"][len(one.colliders):] += len(one.bodies)
    two = scenes.Scene("two worlds", two_b, two_c)
    g, o = make_pair(two)
    g.step(20)
    o.step(20)
    assert_close_rel(g.bodies()["position"], o.bodies()["position"], 1e-5, 1e-5, "positions")
    pr = g.pairs()
    nc1 = len(one.colliders)
    assert len(pr) > 0
    assert not np.any((pr[:, 0] < nc1) & (pr[:, 1] >= nc1))
    np.testing.assert_array_equal(pr, o.pairs())


def test_removal_wakes_the_stack(gpu_lib):
    sc = scenes.pyramid(base=3)
    g, o = make_pair(sc)
    g.step(300)
    o.step(300)
    assert g.bodies()["active"][1:].sum() == 0
    # Remove the ground collider: the bodies touching it wake up and fall.
    h = sc.collider_handles[:1]
    g.remove_colliders(h)
    o.remove_colliders(h)
    g.step(30)
    o.step(30)
    assert g.bodies()["active"][1:].sum() == len(sc.bodies) - 1
    assert_close_rel(g.bodies()["position"], o.bodies()["position"], 1e-5, 1e-5, "positions after removal")


@pytest.mark.parametrize("sched", [abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS])
def test_degenerate_worlds(gpu_lib, sched):
    # Edge cases of the step: a world with no body at all, one with a static
    # ground alone, and one dynamic body falling beside the ground without
    # touching it (no pair, no contact, no solver manifold), under both
    # schedules.
    from nphysics_gb300.world import GpuWorld
    p = abi.default_params()
    p.solver_schedule = sched
    empty = GpuWorld(p)
    empty.step(3)
    assert empty.counters()["num_contacts"] == 0
    g, gc = scenes._ground()
    sc = scenes.Scene("ground alone", *scenes._concat([g], [gc]))
    w = GpuWorld.for_scene(sc, p)
    w.step(3)
    assert w.counters()["num_contacts"] == 0
    b = scenes.body_descs(1)
    b["position"][0, :3] = (500.0, 40.0, 0.0)
    c = scenes.collider_descs(1, 0, abi.SHAPE_BALL, (0.5, 0, 0), density=1.0)
    sc = scenes.Scene("one body", *scenes._concat([g, b], [gc, c]))
    q = sc.params()
    q.solver_schedule = sched
    gw, o = make_pair(sc, q)
    gw.step(20)
    o.step(20)
    assert gw.counters()["num_contacts"] == 0
    np.testing.assert_array_equal(gw.bodies()["position"], o.bodies()["position"])
    np.testing.assert_array_equal(gw.bodies()["velocity"], o.bodies()["velocity"])

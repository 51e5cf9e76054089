"""Compound shapes (ncollide3d Compound) as one collider per part on a body:
the body takes the compound's mass properties (src/volumetric/
volumetric_compound.rs: the parts' masses, centres of mass and inertias
shifted to the common centre and summed) as the reference adds a collider's
(rigid_body.rs:747-766), and each part collides on its own.
The mass properties are checked against the compound formula on the CPU; the
GPU step against the oracle is marked gpu.
"""
import numpy as np
import pytest

from nphysics_gb300 import abi, scenes
from oracle.oracle_py import ORDER_COLOUR, OracleWorld


def _compound_reference(parts, density):
    """volumetric_compound.rs mass_properties for cuboid parts without
    rotation, in f64: the mass, centre and inertia about the centre."""
    ms, cs, Is = [], [], []
    for t, _, shape, h in parts:
        assert shape == abi.SHAPE_CUBOID
        hx, hy, hz = h
        m = density * 8.0 * hx * hy * hz
        ms.append(m)
        cs.append(np.asarray(t, np.float64))
        Is.append(np.diag([m / 3.0 * (hy * hy + hz * hz), m / 3.0 * (hx * hx + hz * hz),
                           m / 3.0 * (hx * hx + hy * hy)]))
    mt = sum(ms)
    com = sum(m * c for m, c in zip(ms, cs)) / mt
    I = np.zeros((3, 3))
    for m, c, Ip in zip(ms, cs, Is):
        d = c - com
        I += Ip + m * (np.dot(d, d) * np.eye(3) - np.outer(d, d))
    return mt, com, I


def _l_shape_scene():
    ident = (0.0, 0.0, 0.0, 1.0)
    parts = [((0.0, 0.0, 0.0), ident, abi.SHAPE_CUBOID, (0.6, 0.15, 0.2)),
             ((0.45, 0.45, 0.0), ident, abi.SHAPE_CUBOID, (0.15, 0.3, 0.2))]
    b = scenes.body_descs(1)
    c, mp = scenes.compound_colliders(0, parts, density=2.5)
    scenes.add_collider_mass(b[0], *mp)
    return scenes.Scene("L", b, c, gravity=(0.0, 0.0, 0.0)), parts


def test_compound_mass_properties_match_the_compound_formula():
    sc, parts = _l_shape_scene()
    o = OracleWorld(sc.params(), sc.gravity, precision=64)
    o.load_scene(sc)
    o.step(1)
    inertia, com = o.mass_properties()
    m, c, I = _compound_reference(parts, 2.5)
    assert inertia[0, 0] == pytest.approx(m, rel=1e-6)
    np.testing.assert_allclose(com[0], c, rtol=0, atol=1e-6)
    got = np.array([[inertia[0, 1], inertia[0, 2], inertia[0, 3]],
                    [inertia[0, 2], inertia[0, 4], inertia[0, 5]],
                    [inertia[0, 3], inertia[0, 5], inertia[0, 6]]])
    np.testing.assert_allclose(got, I, rtol=1e-5, atol=1e-6)


def test_compound_parts_take_the_compound_position():
    # A part's pose on the body is the compound's position times the part's.
    q = np.array([0.0, np.sin(0.3), 0.0, np.cos(0.3)], np.float32)
    parts = [((1.0, 0.0, 0.0), (0.0, 0.0, 0.0, 1.0), abi.SHAPE_BALL, (0.2, 0.0, 0.0))]
    c, (m, com, _) = scenes.compound_colliders(0, parts, position=((0.0, 1.0, 0.0), q), density=1.0)
    p = c["position_wrt_body"][0]
    np.testing.assert_allclose(p[:3], [np.cos(0.6), 1.0, -np.sin(0.6)], atol=1e-6)
    np.testing.assert_allclose(p[3:], q, atol=1e-7)
    # The compound's centre moves with it.
    np.testing.assert_allclose(com, p[:3], atol=1e-6)
    assert m == pytest.approx(4.0 / 3.0 * np.pi * 0.2 ** 3)


def test_compounds_come_to_rest_in_the_oracle():
    sc = scenes.compound_drop()
    o = OracleWorld(sc.params(), sc.gravity, precision=32, order=ORDER_COLOUR)
    o.load_scene(sc)
    o.step(200)
    y = o.bodies()["position"][1:, 1]
    assert (y > 0.05).all() and (y < 0.8).all()


@pytest.mark.gpu
def test_gpu_compounds_match_oracle():
    from nphysics_gb300.world import GpuWorld
    sc = scenes.compound_drop()
    p = sc.params()
    g = GpuWorld.for_scene(sc, p)
    o = OracleWorld(p, sc.gravity, precision=32, order=ORDER_COLOUR)
    o.load_scene(sc)
    for _ in range(150):
        g.step(1)
        o.step(1)
        np.testing.assert_array_equal(g.bodies()["position"], o.bodies()["position"])
    gi, gc = g.mass_properties()
    oi, oc = o.mass_properties()
    np.testing.assert_allclose(gi, oi, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(gc, oc, rtol=1e-6, atol=1e-7)

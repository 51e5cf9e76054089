"""The golden fixtures of tests/golden (made by tests/golden/make_golden.py).

Each fixture holds a scene's input descriptors and what the oracle produced
from them at a few checkpoint steps.

CPU: the scene builders still produce the stored inputs, and the oracle,
re-run on the stored inputs, reproduces every stored output bit for bit (a
regression pin of the restatement and of the fixtures).

GPU: the step through the C ABI, on the stored inputs, reproduces the
colour-order f32 fixtures bit for bit in poses, velocities, activation and
the broad-phase pair set; contact geometry within 1e-5 relative and impulses
within 1e-4 relative (the path's stated bars; in practice they agree bit for
bit too), the contact, solver-contact, colour and awake-body counts exactly,
and the residual, kinetic energy and maximum penetration within 1e-9
relative (FP64 sums taken in another order; the residual's rows in
float-float arithmetic on the GPU).
"""
import glob
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)
import make_golden  # noqa: E402

from oracle.oracle_py import ORDER_COLOUR, ORDER_REFERENCE  # noqa: E402

FIXTURES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
EXACT_COUNTERS = ("num_pairs", "num_contacts", "num_solver_contacts", "num_colours", "num_active_bodies")


def load(name):
    f = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    sc, params, meta = make_golden.scene_from_fixture(f)
    return f, sc, params, meta


def test_every_case_has_a_fixture():
    assert FIXTURES == sorted(make_golden.CASES)


@pytest.mark.parametrize("name", FIXTURES)
def test_scene_builders_reproduce_stored_inputs(name):
    f, sc, params, meta = load(name)
    assert meta["format"] == make_golden.FORMAT
    assert meta["body_itemsize"] == sc.bodies.dtype.itemsize
    assert meta["collider_itemsize"] == sc.colliders.dtype.itemsize
    built = make_golden.CASES[name][0]()
    assert np.ascontiguousarray(built.bodies).tobytes() == f["bodies_raw"].tobytes()
    assert np.ascontiguousarray(built.colliders).tobytes() == f["colliders_raw"].tobytes()
    assert make_golden.params_delta(built.params()) == meta["params"]


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_reproduces_fixture(name):
    f, sc, params, meta = load(name)
    order = ORDER_COLOUR if meta["order"] == "colour" else ORDER_REFERENCE
    out = make_golden.run_oracle(sc, params, meta["precision"], order, meta["checkpoints"])
    assert sorted(out) == sorted(k for k in f.files if k not in ("meta", "bodies_raw", "colliders_raw"))
    for k, v in out.items():
        assert v.dtype == f[k].dtype, k
        np.testing.assert_array_equal(v, f[k], err_msg=f"{name}: {k}")


def test_fixtures_exercise_contacts():
    # Every fixture reaches contact, and the set covers box-box, ball-box and
    # ball-ball manifolds, several colours, and both precisions and orders.
    kinds = set()
    for name in FIXTURES:
        f, sc, _, meta = load(name)
        last = meta["checkpoints"][-1]
        c = dict(zip(meta["counter_keys"], f[f"counters_{last}"]))
        assert c["num_contacts"] > 50, name
        kinds.add((meta["precision"], meta["order"]))
        shape = sc.colliders["shape"]
        k1 = f[f"contact_key_{last}"] >> np.uint64(40)
        k2 = (f[f"contact_key_{last}"] >> np.uint64(10)) & np.uint64((1 << 30) - 1)
        for a, b in zip(shape[k1.astype(np.int64)], shape[k2.astype(np.int64)]):
            kinds.add(tuple(sorted((int(a), int(b)))))
    assert {(32, "colour"), (64, "reference")} <= kinds
    assert len([k for k in kinds if isinstance(k[1], int)]) == 3


def _rel_close(a, b, rtol, atol, what):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    err = np.abs(a - b)
    bad = err > atol + rtol * np.abs(b)
    assert not bad.any(), f"{what}: {bad.sum()} of {bad.size} beyond tolerance; max err {err.max():.3e}"


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in FIXTURES if not n.endswith("_f64_reference")])
def test_gpu_reproduces_fixture(gpu_lib, name):
    from nphysics_gb300.world import GpuWorld
    f, sc, params, meta = load(name)
    assert meta["precision"] == 32 and meta["order"] == "colour"
    g = GpuWorld.for_scene(sc, params)
    done = 0
    for s in meta["checkpoints"]:
        g.step(s - done)
        done = s
        b = g.bodies()
        np.testing.assert_array_equal(b["position"].astype(np.float32), f[f"position_{s}"], err_msg=f"{name} @{s}")
        np.testing.assert_array_equal(b["velocity"].astype(np.float32), f[f"velocity_{s}"], err_msg=f"{name} @{s}")
        np.testing.assert_array_equal(b["active"], f[f"active_{s}"], err_msg=f"{name} @{s}")
        np.testing.assert_array_equal(g.pairs(), f[f"pairs_{s}"], err_msg=f"{name} @{s}")
        key, c = make_golden.contact_table(g.contacts())
        np.testing.assert_array_equal(key, f[f"contact_key_{s}"], err_msg=f"{name} @{s}")
        for k in ("world1", "world2", "normal", "depth"):
            _rel_close(c[k], f[f"contact_{k}_{s}"], 1e-5, 1e-5, f"{name} @{s}: {k}")
        _rel_close(c["impulse"], f[f"contact_impulse_{s}"], 1e-4, 1e-6, f"{name} @{s}: impulse")
        cg = g.counters()
        co = dict(zip(meta["counter_keys"], f[f"counters_{s}"]))
        for k in EXACT_COUNTERS:
            assert cg[k] == co[k], (name, s, k, cg[k], co[k])
        for k in ("residual", "kinetic_energy", "max_penetration"):
            assert abs(cg[k] - co[k]) <= 1e-9 * abs(co[k]) + 1e-15, (name, s, k, cg[k], co[k])
    g.close()

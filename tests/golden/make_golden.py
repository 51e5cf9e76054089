"""Generates the golden fixtures of this directory from the CPU oracle.

Each fixture is self-contained: the scene's input descriptors (the raw bytes
of npgpu_body_desc / npgpu_collider_desc arrays), gravity and the parameters
that differ from IntegrationParameters::default(), then what the oracle
produced at a few checkpoint steps: body poses, velocities and activation,
the broad-phase pair set, the contact table (sorted by collider pair and
feature key) and the step counters.

Run from the repository root:

    python tests/golden/make_golden.py

The oracle is the only producer. The reference (nphysics3d, a Rust crate)
cannot be built on this machine, so these vectors pin the restatement and
the GPU against each other, not against nphysics itself; the reference's own
known-answer test (the cuboid mass properties of
src/volumetric/volumetric_convex3.rs:285-346) is checked in test_oracle_kat.py.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from nphysics_gb300 import abi, scenes  # noqa: E402
from oracle.oracle_py import ORDER_COLOUR, ORDER_REFERENCE, OracleWorld  # noqa: E402

FORMAT = 1

# name -> (scene builder, precision, Gauss-Seidel order, checkpoint steps)
CASES = {
    "pyramid_base6": (lambda: scenes.pyramid(base=6), 32, ORDER_COLOUR, (1, 20, 120)),
    "ball_pile_side5": (lambda: scenes.ball_pile(side=5), 32, ORDER_COLOUR, (1, 30, 90)),
    "cluster_64": (lambda: scenes.random_cluster(n=64, seed=7, extent=3.0), 32, ORDER_COLOUR, (1, 10, 40)),
    "mixed_300": (lambda: scenes.mixed_lattice(n=300, seed=5, footprint=12.0), 32, ORDER_COLOUR, (1, 90, 200)),
    "batched_6": (lambda: scenes.batched_worlds(n_worlds=6, seed=3, lo=8, hi=120), 32, ORDER_COLOUR, (1, 25)),
    "brick_walls_2x48": (lambda: scenes.brick_walls(n_walls=2, width=8, height=6, balls=3, seed=5), 32, ORDER_COLOUR,
                         (1, 60, 150)),
    "pyramid_base6_f64_reference": (lambda: scenes.pyramid(base=6), 64, ORDER_REFERENCE, (1, 120)),
}

COUNTER_KEYS = ("num_pairs", "num_manifolds", "num_contacts", "num_solver_contacts", "num_constraints",
                "num_colours", "num_active_bodies", "velocity_iterations", "residual", "max_penetration",
                "kinetic_energy")
CONTACT_FIELDS = ("world1", "world2", "normal", "depth", "impulse", "colour")


def params_delta(p):
    """The fields of p that differ from abi.default_params(), by name."""
    d = abi.default_params()
    out = {}
    for name, _ in abi.Params._fields_:
        a, b = getattr(p, name), getattr(d, name)
        if a != b:
            out[name] = a
    return out


def params_from_delta(delta):
    p = abi.default_params()
    for k, v in delta.items():
        setattr(p, k, v)
    return p


def scene_from_fixture(f):
    """The Scene stored in a loaded fixture."""
    meta = json.loads(str(f["meta"]))
    bodies = np.frombuffer(f["bodies_raw"].tobytes(), scenes.BODY_DTYPE).copy()
    colliders = np.frombuffer(f["colliders_raw"].tobytes(), scenes.COLLIDER_DTYPE).copy()
    assert len(bodies) == meta["num_bodies"] and len(colliders) == meta["num_colliders"]
    sc = scenes.Scene(meta["name"], bodies, colliders, gravity=meta["gravity"], dt=meta["params"].get("dt", 1 / 60))
    return sc, params_from_delta(meta["params"]), meta


def contact_table(c):
    """Contacts sorted by (collider1, collider2, feature key)."""
    key = (c["collider1"].astype(np.uint64) << np.uint64(40)) | (c["collider2"].astype(np.uint64) << np.uint64(10)) | \
        c["feature_key"].astype(np.uint64)
    order = np.argsort(key, kind="stable")
    return key[order], {k: v[order] for k, v in c.items()}


def run_oracle(scene, params, precision, order, checkpoints):
    """Steps the oracle through the checkpoints; returns the arrays to store."""
    w = OracleWorld(params, scene.gravity, precision=precision, order=order)
    w.load_scene(scene)
    out = {}
    dt_out = np.float32 if precision == 32 else np.float64
    done = 0
    for s in checkpoints:
        w.step(s - done)
        done = s
        b = w.bodies()
        out[f"position_{s}"] = b["position"].astype(dt_out)
        out[f"velocity_{s}"] = b["velocity"].astype(dt_out)
        out[f"active_{s}"] = b["active"].copy()
        out[f"pairs_{s}"] = w.pairs()
        key, c = contact_table(w.contacts())
        out[f"contact_key_{s}"] = key
        for k in CONTACT_FIELDS:
            out[f"contact_{k}_{s}"] = c[k]
        cn = w.counters()
        out[f"counters_{s}"] = np.array([cn[k] for k in COUNTER_KEYS], np.float64)
    w.close()
    return out


def make(name):
    build, precision, order, checkpoints = CASES[name]
    sc = build()
    p = sc.params()
    arrays = run_oracle(sc, p, precision, order, checkpoints)
    meta = {
        "format": FORMAT, "name": name, "precision": precision,
        "order": "colour" if order == ORDER_COLOUR else "reference",
        "checkpoints": list(checkpoints), "gravity": list(sc.gravity), "params": params_delta(p),
        "num_bodies": int(len(sc.bodies)), "num_colliders": int(len(sc.colliders)),
        "body_itemsize": scenes.BODY_DTYPE.itemsize, "collider_itemsize": scenes.COLLIDER_DTYPE.itemsize,
        "counter_keys": list(COUNTER_KEYS),
    }
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), meta=np.array(json.dumps(meta)),
                        bodies_raw=np.frombuffer(np.ascontiguousarray(sc.bodies).tobytes(), np.uint8),
                        colliders_raw=np.frombuffer(np.ascontiguousarray(sc.colliders).tobytes(), np.uint8),
                        **arrays)


if __name__ == "__main__":
    for n in (sys.argv[1:] or CASES):
        make(n)
        print("wrote", n)

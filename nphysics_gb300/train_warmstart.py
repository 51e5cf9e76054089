"""Trains the learned warm start on a scene and saves the network.

The GPU world steps the scene with the velocity solver run to a tight
residual, recording every solver contact (features at assembly, converged
impulses after the solve). The recorded samples then train the network on
the GPU (npgpu_mlp_train). The saved parameters (NPGPU_MLP_PARAMS float32
values) load with GpuWorld.mlp_set / npgpu_mlp_set.

    python -m nphysics_gb300.train_warmstart --scene mixed --size 20000 \\
        --record-steps 300 --train-steps 3000 --out warmstart.npy

With --evaluate-steps K, the scene is then run again from its start with the
impulse cache alone and with the trained network, K steps each, at 8
iterations and solved to 1e-3 and to 1e-4 (at most 256 iterations), and one
JSON line per run reports the mean iterations and residuals.

With --ablation, the 100k mixed pile is the workload: samples are recorded
on it (one step in 30 of a 300-step settle, each solved to 1e-5), then every
variant is evaluated from the same settled state (300 steps at the default 8
iterations), solving 10 steps to 1e-4: the zero start, the impulse cache,
the network for new contacts (mode 2) and for every contact (mode 3), and
mode 3 with each feature group left out of training (its columns zeroed, so
that normalisation gives them zero weight). One JSON line per variant.

    python -m nphysics_gb300.train_warmstart --ablation
"""
import argparse
import json
import time

import numpy as np

from . import abi, scenes
from .world import GpuWorld


def make_scene(kind, size):
    if kind == "pile":
        return scenes.ball_pile(side=size)
    if kind == "mixed":
        return scenes.mixed_pile(n=size)
    if kind == "pyramid":
        return scenes.pyramid(base=size)
    raise ValueError(f"unknown scene {kind}")


def record(scene, steps, tolerance, capacity, max_iterations=256):
    p = scene.params()
    p.solve_to_tolerance = 1
    p.residual_tolerance = tolerance
    p.max_iterations_to_tolerance = max_iterations
    w = GpuWorld.for_scene(scene, p)
    w.mlp_record(capacity)
    w.step(steps)
    w.mlp_record(0)
    return w


def evaluate(scene_fn, net, steps, warmstart_mode, tolerance=None, iterations=8):
    """Mean iterations, residuals and learned-start counts over `steps` steps
    of a fresh world (steps without solver contacts are left out)."""
    sc = scene_fn()
    p = sc.params()
    p.warmstart_mode = warmstart_mode
    if tolerance:
        p.solve_to_tolerance = 1
        p.residual_tolerance = tolerance
        p.max_iterations_to_tolerance = 256
    else:
        p.max_velocity_iterations = iterations
    w = GpuWorld.for_scene(sc, p)
    if warmstart_mode == abi.WARMSTART_LEARNED:
        w.mlp_set(net)
    its, r0, r1, starts, kept = [], [], [], 0, 0
    for _ in range(steps):
        w.step(1)
        c = w.counters()
        if c["num_solver_contacts"] == 0:
            continue
        its.append(c["velocity_iterations"])
        r0.append(c["residual_initial"])
        r1.append(c["residual"])
        starts += c["learned_starts"]
        kept += c["learned_kept"]
    return {"warmstart": {abi.WARMSTART_CACHE: "cache", abi.WARMSTART_LEARNED: "learned"}[warmstart_mode],
            "tolerance": tolerance, "iterations": None if tolerance else iterations, "steps": len(its),
            "iterations_mean": float(np.mean(its)) if its else 0.0,
            "residual_after_warm_start": float(np.mean(r0)) if r0 else 0.0,
            "residual_final": float(np.mean(r1)) if r1 else 0.0, "learned_starts": starts, "learned_kept": kept}


FEATURE_GROUPS = {
    "rows_rhs_and_r": list(range(0, 6)),
    "depth": [6],
    "masses_and_angular_terms": list(range(7, 15)),
    "friction_and_gravity": [15, 16, 23],
    "contact_and_manifold_counts": [17, 18, 19],
    "one_row_solutions": [20, 21, 22],
}


def _settled(scene, settle):
    w = GpuWorld.for_scene(scene, scene.params(), pairs_per_collider=12)
    w.step(settle)
    return w


def _solve_to(w, mode, net, steps, tolerance=1e-4, cap=4096):
    if net is not None:
        w.mlp_set(net)
    p = w.params
    p.warmstart_mode = mode
    p.solve_to_tolerance = 1
    p.residual_tolerance = tolerance
    p.max_iterations_to_tolerance = cap
    w.set_params(p)
    its, r0, starts, kept = [], [], 0, 0
    for _ in range(steps):
        w.step(1)
        c = w.counters()
        its.append(c["velocity_iterations"])
        r0.append(c["residual_initial"])
        starts += c["learned_starts"]
        kept += c["learned_kept"]
    return {"iterations_mean": float(np.mean(its)), "iterations_max": int(np.max(its)),
            "residual_after_warm_start": float(np.mean(r0)), "learned_starts": starts, "learned_kept": kept}


def ablation(settle=300, steps=10, train_steps=4000):
    """Variants of the warm start on the 100k mixed pile (see the module text)."""
    scene = scenes.mixed_pile(n=100_000)
    rec = _settled(scene, 60)
    parts = []
    p = rec.params
    for k in range(9):
        p.solve_to_tolerance, p.residual_tolerance, p.max_iterations_to_tolerance = 1, 1e-5, 1024
        rec.set_params(p)
        rec.mlp_record(4_000_000)
        rec.step(1)
        parts.append(rec.mlp_samples())
        rec.mlp_record(0)
        p.solve_to_tolerance = 0
        rec.set_params(p)
        rec.step(29)
    samples = np.concatenate(parts)
    rng = np.random.default_rng(5)
    samples = samples[rng.choice(len(samples), min(len(samples), 2_000_000), replace=False)]

    def train(columns_out=()):
        s = samples.copy()
        if columns_out:
            s[:, list(columns_out)] = 0.0
        rec.mlp_load_samples(s)
        rec.mlp_train(1, batch=4096, lr=1e-3, seed=1, init=True)
        loss = rec.mlp_train(train_steps, batch=4096, lr=1e-3, seed=2)
        return rec.mlp_get(), loss

    out = []
    for name, mode in (("zero start", abi.WARMSTART_NONE), ("impulse cache", abi.WARMSTART_CACHE)):
        w = _settled(scene, settle)
        out.append(dict({"variant": name}, **_solve_to(w, mode, None, steps)))
        w.close()
    net, loss = train()
    for name, mode in (("network, new contacts (mode 2)", abi.WARMSTART_LEARNED),
                       ("network, every contact (mode 3)", abi.WARMSTART_LEARNED_ALL)):
        w = _settled(scene, settle)
        out.append(dict({"variant": name, "loss": loss}, **_solve_to(w, mode, net, steps)))
        w.close()
    for group, cols in FEATURE_GROUPS.items():
        net_g, loss_g = train(cols)
        w = _settled(scene, settle)
        out.append(dict({"variant": f"mode 3 without {group}", "loss": loss_g},
                        **_solve_to(w, abi.WARMSTART_LEARNED_ALL, net_g, steps)))
        w.close()
    rec.close()
    for r in out:
        r["samples"] = len(samples)
        print(json.dumps(r), flush=True)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--scene", default="mixed", choices=["pile", "mixed", "pyramid"])
    ap.add_argument("--size", type=int, default=20000,
                    help="balls per side (pile), bodies (mixed) or base boxes (pyramid)")
    ap.add_argument("--record-steps", type=int, default=300)
    ap.add_argument("--tolerance", type=float, default=1e-5)
    ap.add_argument("--capacity", type=int, default=4_000_000)
    ap.add_argument("--train-steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=None, help="where to save the parameters (.npy)")
    ap.add_argument("--evaluate-steps", type=int, default=0)
    ap.add_argument("--ablation", action="store_true", help="the warm-start ablation on the 100k mixed pile")
    args = ap.parse_args(argv)
    if args.ablation:
        ablation()
        return

    t0 = time.perf_counter()
    w = record(make_scene(args.scene, args.size), args.record_steps, args.tolerance, args.capacity)
    n = w.mlp_samples(download=False)
    t1 = time.perf_counter()
    first = w.mlp_train(1, batch=args.batch, lr=args.lr, seed=args.seed, init=True)
    last = w.mlp_train(args.train_steps, batch=args.batch, lr=args.lr, seed=args.seed + 1)
    t2 = time.perf_counter()
    if args.out:
        np.save(args.out, w.mlp_get())
    print(json.dumps({"samples": n, "record_s": t1 - t0, "train_s": t2 - t1, "loss_first": first,
                      "loss_last": last, "out": args.out}), flush=True)
    if args.evaluate_steps:
        net = w.mlp_get()
        del w
        for tol in (None, 1e-3, 1e-4):
            for mode in (abi.WARMSTART_CACHE, abi.WARMSTART_LEARNED):
                r = evaluate(lambda: make_scene(args.scene, args.size), net, args.evaluate_steps, mode, tol)
                print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main()

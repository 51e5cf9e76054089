"""One step of a workload inside a profiler range, for ncu captures.

The workload is built and stepped untimed to the state the benchmark times
(settle steps, then a few more), then exactly one region runs between
cudaProfilerStart and cudaProfilerStop, so that

    ncu --profile-from-start off --clock-control none --metrics ... \\
        python -m nphysics_gb300.profile_step --workload pile

captures that region's launches and nothing else. Regions:

  step      one npgpu_step of the workload (every kernel of the step)
  e2e       one end-to-end round trip through the C ABI: npgpu_apply_forces
            from page-locked host arrays, npgpu_step, npgpu_download_bodies
  train     --train-steps Adam steps of the learned warm start on samples the
            workload's solver recorded (the network's kernels)

Workloads: pile (the 32^3 ball pile, one cooperative grid), cluster (the same
pile under the per-world schedule: one thread-block cluster), batched
(--worlds batched worlds, one block or warp per world), mixed (--bodies
bodies of the mixed pile's recipe at its density).
"""
import argparse
import math

import numpy as np


def pinned(a):
    """A copy of `a` in page-locked host memory (a numpy view of a pinned torch buffer)."""
    import torch
    buf = torch.empty(max(a.nbytes, 1), dtype=torch.uint8, pin_memory=True).numpy()
    out = buf[:a.nbytes].view(a.dtype).reshape(a.shape)
    out[...] = a
    return out


def build(args):
    from . import abi, scenes
    from .world import GpuWorld
    if args.workload in ("pile", "cluster"):
        sc = scenes.ball_pile(side=args.side)
        p = sc.params()
        p.solver_schedule = abi.SCHEDULE_WORLDS if args.workload == "cluster" else abi.SCHEDULE_GRID
        return sc, GpuWorld.for_scene(sc, p), 200
    if args.workload == "batched":
        sc = scenes.batched_worlds(n_worlds=args.worlds)
        p = sc.params()
        p.solver_schedule = abi.SCHEDULE_WORLDS
        p.world_threads = 256
        return sc, GpuWorld.for_scene(sc, p, pairs_per_collider=6), 60
    n = args.bodies
    sc = scenes.mixed_pile(n=n, footprint=100.0 * math.sqrt(n / 100_000))
    return sc, GpuWorld.for_scene(sc, sc.params(), pairs_per_collider=12), 300


def main(argv=None):
    import torch

    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--workload", default="pile", choices=["pile", "cluster", "batched", "mixed"])
    ap.add_argument("--region", default="step", choices=["step", "e2e", "train"])
    ap.add_argument("--side", type=int, default=32)
    ap.add_argument("--worlds", type=int, default=1024)
    ap.add_argument("--bodies", type=int, default=100_000)
    ap.add_argument("--settle", type=int, default=None)
    ap.add_argument("--train-steps", type=int, default=3)
    args = ap.parse_args(argv)

    from . import build as nb
    nb.build()
    torch.cuda.init()
    sc, w, settle = build(args)
    w.step(args.settle if args.settle is not None else settle)
    w.step(3)      # graphs captured, caches warm
    if args.region == "train":
        p = w.params
        p.solve_to_tolerance, p.residual_tolerance, p.max_iterations_to_tolerance = 1, 1e-5, 256
        w.set_params(p)
        w.mlp_record(1_000_000)
        w.step(1)
        w.mlp_record(0)
        w.mlp_train(1, batch=4096, lr=1e-3, seed=1, init=True)
    pos = vel = handles = forces = None
    if args.region == "e2e":
        pos = pinned(np.zeros((len(sc.bodies), 7), np.float32))
        vel = pinned(np.zeros((len(sc.bodies), 6), np.float32))
        dyn = np.nonzero(sc.bodies["status"] == 2)[0]
        handles = pinned(np.ascontiguousarray(sc.body_handles[dyn]))
        forces = pinned(np.zeros((len(dyn), 6), np.float32))
        w.apply_forces(handles, forces, wake=False)
        w.step(1, sync=False)
        w.download_into(pos, vel)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    if args.region == "step":
        w.step(1)
    elif args.region == "e2e":
        w.apply_forces(handles, forces, wake=False)
        w.step(1, sync=False)
        w.download_into(pos, vel)
    else:
        w.mlp_train(args.train_steps, batch=4096, lr=1e-3, seed=2)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    c = w.counters()
    print(f"profiled {args.region} of {sc.name}: {c['num_contacts']} contacts, {c['num_colours']} colours, "
          f"{sc.num_dynamic} dynamic bodies")
    w.close()


if __name__ == "__main__":
    main()

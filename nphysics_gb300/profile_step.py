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
  train     the learned warm start trained on samples the workload's solver
            recorded: normalisation and initialisation, then --train-steps
            Adam steps (the network's kernels)
  query     one batch each of --queries rays, points and boxes against the
            world (interferences_with_ray / _point / _aabb)
  events    one step with contact events recorded
  static    the allocation-free pair finder on the world's fat AABBs

Workloads: pile (the 32^3 ball pile, one cooperative grid), cluster (the same
pile under the per-world schedule: one thread-block cluster), batched
(--worlds batched worlds, one block or warp per world), mixed (--bodies
bodies of the mixed pile's recipe at its density), joints (--worlds worlds
of every joint kind with contacts), walls_ccd (--worlds brick walls struck by
balls with CCD, from step 60 when the balls reach the walls).
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
    if args.workload == "joints":
        # Worlds of every joint kind with contacts, one block (or warp) per world.
        sc = scenes.batched_zoo(n_worlds=args.worlds)
        return sc, GpuWorld.for_scene(sc), 60
    if args.workload == "walls_ccd":
        sc = scenes.brick_walls(n_walls=args.worlds, ccd=True)
        return sc, GpuWorld.for_scene(sc, sc.params(), pairs_per_collider=8), 60
    n = args.bodies
    sc = scenes.mixed_pile(n=n, footprint=100.0 * math.sqrt(n / 100_000))
    return sc, GpuWorld.for_scene(sc, sc.params(), pairs_per_collider=12), 300


def main(argv=None):
    import torch

    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--workload", default="pile",
                    choices=["pile", "cluster", "batched", "mixed", "joints", "walls_ccd"])
    ap.add_argument("--region", default="step", choices=["step", "e2e", "train", "query", "events", "static"])
    ap.add_argument("--queries", type=int, default=100_000)
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
    rng = np.random.default_rng(1)
    if args.region == "query":
        lo, hi = sc.bodies["position"][:, :3].min(axis=0), sc.bodies["position"][:, :3].max(axis=0)
        org = rng.uniform(lo, hi, (args.queries, 3)).astype(np.float32)
        rays = np.concatenate([org, rng.normal(size=(args.queries, 3)).astype(np.float32)], axis=1)
        toi = np.full(args.queries, 5.0, np.float32)
        boxes = np.concatenate([org, org + 1.0], axis=1)
    if args.region == "events":
        w.enable_contact_events(1 << 20)
        w.step(1)
    if args.region == "static":
        from . import abi
        import ctypes as C
        aabbs = torch.from_numpy(w.aabbs()).cuda()
        n = min(len(aabbs), 32768)
        pairs = torch.empty((16 * n, 2), dtype=torch.int32, device="cuda")
        count = torch.empty(1, dtype=torch.int32, device="cuda")
        args_static = (C.c_void_p(aabbs.data_ptr()), None, n, C.c_void_p(pairs.data_ptr()), 16 * n,
                       C.c_void_p(count.data_ptr()), None)
        assert w.L.npgpu_find_pairs_static(*args_static) == abi.OK     # set-up call
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    if args.region in ("step", "events"):
        w.step(1)
    elif args.region == "query":
        w.rays(rays, toi)
        w.points(org)
        w.aabb_query(boxes)
    elif args.region == "static":
        w.L.npgpu_find_pairs_static(*args_static)
    elif args.region == "e2e":
        w.apply_forces(handles, forces, wake=False)
        w.step(1, sync=False)
        w.download_into(pos, vel)
    else:
        w.mlp_train(1, batch=4096, lr=1e-3, seed=1, init=True)
        w.mlp_train(args.train_steps, batch=4096, lr=1e-3, seed=2)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    c = w.counters()
    print(f"profiled {args.region} of {sc.name}: {c['num_contacts']} contacts, {c['num_colours']} colours, "
          f"{sc.num_dynamic} dynamic bodies")
    w.close()


if __name__ == "__main__":
    main()

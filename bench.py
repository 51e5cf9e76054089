"""Benchmark of the GPU rigid-body step: body-steps/s on the 32^3 ball pile.

Workload: 32768 balls of radius 0.5 on a 1.2 lattice (seeded jitter),
dropped on a static ground, density 1, friction 0.3, dt 1/60, the
reference's 8 velocity / 3 position iterations. The pile is simulated
untimed for --settle steps (it reaches the ground and forms contacts), then
--warmup steps, then --steps timed steps.

  value  body-steps/s with the world resident in HBM: CUDA events on the
         world's stream around each step, an L2 flush (256 MiB write)
         between steps, outside the timed region.
  e2e    the same metric through the C ABI as a host would drive it: per
         step, upload of the step's applied forces from pinned host memory,
         npgpu_step, download of every body's pose and velocity into host
         buffers; wall time of the loop.
  pgs_iterations  the metric's second half on the same pile: mean SOR-Prox
         iterations to a residual of 1e-4, impulse cache alone vs the learned
         warm start (network trained in the run on the solver's own impulses).
  --impl reference  times the CPU oracle (the restated reference step) on
         this host instead (the Rust reference cannot be built here).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "body-steps/s"
L2_FLUSH_BYTES = 256 << 20
PROFILE_STEPS = 10
# Kernels of this library launched per step (CUB's radix sort and scans not
# counted), from the ncu launch list of this workload.
LAUNCHES_PER_STEP = 21
# The per-world schedule: the two cooperative solver kernels become seven
# per-world kernels (bucket count and scatter, the two renumbering passes,
# velocity, residual, position), from the launch list of the batched workload.
LAUNCHES_PER_STEP_BATCHED = 26
# dram__bytes_read.sum + dram__bytes_write.sum of one k_velocity launch on this
# workload, from one ncu capture.
VELOCITY_TRAFFIC_PER_LAUNCH = 45684480
# dram__bytes_read.sum + dram__bytes_write.sum of one k_world_velocity launch
# on a 1024-world batch (1 057 024 solver contacts), per solver contact: the
# batched line scales it by its own solver contacts (the traffic of the
# per-world kernel grows with the contacts it sweeps).
WORLD_VELOCITY_TRAFFIC_PER_CONTACT = 580477184 / 1057024


def pinned(a):
    """A copy of `a` in page-locked host memory (a numpy view of a pinned torch buffer)."""
    import torch
    buf = torch.empty(max(a.nbytes, 1), dtype=torch.uint8, pin_memory=True).numpy()
    out = buf[:a.nbytes].view(a.dtype).reshape(a.shape)
    out[...] = a
    return out


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--settle", type=int, default=None,
                    help="untimed steps first (default: 200 for the ball pile and the pyramid, 150 for the mixed "
                         "pile, 60 for batched worlds, 0 for the brick walls, whose impact phase is the workload)")
    ap.add_argument("--side", type=int, default=32)
    ap.add_argument("--workload", default="pile", choices=["pile", "batched", "pyramid", "walls", "mixed"],
                    help="pile: the 32^3 ball pile (replicas on N GPUs); batched: --worlds-per-rank worlds "
                         "of the batched-worlds scene per GPU (the batch sharded across ranks); pyramid: the "
                         "210-box pyramid (replicas); walls: 256 brick walls struck by balls per GPU; mixed: "
                         "the 100k pile of balls and cuboids (replicas)")
    ap.add_argument("--worlds-per-rank", type=int, default=4096)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--schedule", default="auto", choices=["auto", "grid", "worlds"],
                    help="solver launch shape: timed candidates (auto), the one cooperative grid, or one "
                         "block or warp per world (batched worlds)")
    ap.add_argument("--world-threads", type=int, default=256, choices=[64, 128, 256],
                    help="threads per block of the per-world schedule when --schedule worlds")
    ap.add_argument("--no-pgs-iterations", action="store_true",
                    help="skip the iterations-to-1e-4 comparison of the learned and plain warm starts")
    args = ap.parse_args()
    if args.settle is None:
        args.settle = {"pile": 200, "batched": 60, "pyramid": 200, "walls": 0, "mixed": 150}[args.workload]
    return args


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_sample(scene_fn, settle_steps, max_steps, seconds):
    """Times the oracle (the restated reference step, f32, one thread, the
    reference's row order) on a bounded sample of the same workload: the pile
    is settled for `settle_steps` untimed steps, exactly as on the GPU, then
    up to `max_steps` steps are timed, stopping after about `seconds`."""
    from oracle.oracle_py import ORDER_REFERENCE, OracleWorld
    sc = scene_fn()
    o = OracleWorld(sc.params(), sc.gravity, precision=32, order=ORDER_REFERENCE)
    o.load_scene(sc)
    o.step(settle_steps)
    steps = 0
    t0 = time.perf_counter()
    while steps < max_steps and (steps == 0 or time.perf_counter() - t0 < seconds):
        o.step(1)
        steps += 1
    dt = time.perf_counter() - t0
    c = o.counters()
    sample = (f"steps {settle_steps}..{settle_steps + steps - 1} of the same {sc.num_dynamic}-ball pile "
              f"({c['num_contacts']} contacts), single-threaded f32 oracle in the reference's row order; "
              "the Rust reference has no toolchain on this host")
    return sc.num_dynamic * steps / dt, steps, dt, sample


def cpu_baseline(scene_fn, seconds, settle_steps):
    value, steps, dt, sample = cpu_sample(scene_fn, settle_steps, 10 ** 9, seconds)
    return {"value": value, "unit": METRIC, "cores": 1, "kind": "port", "sample": sample}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from nphysics_gb300 import scenes
    n_dyn = args.side ** 3
    value, steps, dt, sample = cpu_sample(lambda: scenes.ball_pile(side=args.side), args.settle + args.warmup,
                                          args.steps, max(5.0, args.cpu_seconds))
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"ball pile {args.side}^3 = {n_dyn} balls (radius 0.5, 1.2 lattice, seeded jitter) "
                               f"on a static ground, dt 1/60, 8 velocity / 3 position iterations; timed steps "
                               f"{args.settle + args.warmup}..{args.settle + args.warmup + steps - 1} of the run",
                   "sample": sample},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": 1, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def pgs_iterations(scene_fn, settle, steps=30, record_steps=100, train_steps=2000):
    """The metric's second half on the same workload: mean SOR-Prox iterations
    to a residual of 1e-4 (at most 256), with the impulse cache alone and
    with the learned warm start. The network is trained in this run on the
    solver's own converged impulses of the workload (record_steps steps solved
    to 1e-5). Both worlds are stepped `settle` steps with the default
    parameters first, so they start the comparison from the same bits."""
    from nphysics_gb300 import abi
    from nphysics_gb300.train_warmstart import record
    t0 = time.perf_counter()
    rec = record(scene_fn(), record_steps, 1e-5, 4_000_000)
    n_samples = rec.mlp_samples(download=False)
    rec.mlp_train(1, batch=4096, lr=1e-3, seed=1, init=True)
    loss = rec.mlp_train(train_steps, batch=4096, lr=1e-3, seed=2)
    net = rec.mlp_get()
    rec.close()
    out = {"tolerance": 1e-4, "max_iterations": 256, "steps": steps,
           "network": f"trained in this run: {n_samples} samples from {record_steps} steps solved to 1e-5, "
                      f"{train_steps} Adam steps (batch 4096, lr 1e-3), final loss {loss:.3f}"}
    from nphysics_gb300.world import GpuWorld
    for name, mode in (("plain", abi.WARMSTART_CACHE), ("learned", abi.WARMSTART_LEARNED)):
        sc = scene_fn()
        w = GpuWorld.for_scene(sc, sc.params())
        w.mlp_set(net)
        w.step(settle)
        p = w.params
        p.warmstart_mode = mode
        p.solve_to_tolerance = 1
        p.residual_tolerance = 1e-4
        p.max_iterations_to_tolerance = 256
        w.set_params(p)
        its, r0, ms = [], [], []
        for _ in range(steps):
            a = time.perf_counter()
            w.step(1)
            ms.append(time.perf_counter() - a)
            c = w.counters()
            its.append(c["velocity_iterations"])
            r0.append(c["residual_initial"])
        out[name] = {"iterations_mean": statistics.mean(its), "residual_after_warm_start": statistics.mean(r0),
                     "body_steps_per_s": sc.num_dynamic * steps / sum(ms)}
        w.close()
    out["seconds"] = time.perf_counter() - t0
    return out


def run_gpu(args):
    import numpy as np
    import torch

    from nphysics_gb300 import build, scenes
    from nphysics_gb300.world import GpuWorld

    from nphysics_gb300 import multirank
    rank, world_size, local_rank = multirank.rank_env()
    torch.cuda.set_device(local_rank)
    if world_size > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build.build()
    torch.cuda.init()
    if args.workload == "pile":
        # Replicas: every rank runs its own copy of the pile (one world per GPU).
        sc = scenes.ball_pile(side=args.side)
        w = GpuWorld.for_scene(sc, sc.params())
        workload = (f"ball pile {args.side}^3 = {sc.num_dynamic} balls (radius 0.5, 1.2 lattice, seeded jitter) "
                    f"on a static ground, dt 1/60, 8 velocity / 3 position iterations")
    elif args.workload == "pyramid":
        sc = scenes.pyramid(base=20)
        w = GpuWorld.for_scene(sc, sc.params())
        workload = ("box pyramid: 210 cuboids of half extent 0.5 in a 20-base triangle on a static ground, "
                    "density 1, friction 0.5, dt 1/60, 8 velocity / 3 position iterations")
    elif args.workload == "mixed":
        # Replicas: the 100k mixed pile of balls and cuboids on every rank.
        sc = scenes.mixed_pile(n=100_000)
        w = GpuWorld.for_scene(sc, sc.params(), pairs_per_collider=12)
        workload = ("mixed pile: 100000 bodies, half balls of radius U(0.2, 0.8), half cuboids of half extents "
                    "U(0.2, 0.8)^3 at random orientations, density 1, friction 0.5, dropped from a jittered 2.0 "
                    "lattice onto a static ground, dt 1/60, 8 velocity / 3 position iterations")
    elif args.workload == "walls":
        # Each rank steps its own 256 walls (weak scaling).
        sc = scenes.brick_walls(n_walls=256, seed=1234 + rank)
        w = GpuWorld.for_scene(sc, sc.params(), pairs_per_collider=8)
        workload = ("brick walls: 256 walls per GPU of 50 x 40 bricks (half extents 0.5 x 0.25 x 0.25, running "
                    "bond), each struck by 64 balls of radius 0.4, density 10, at U(20, 40) m/s; friction 0.6, "
                    "dt 1/120, 8 velocity / 3 position iterations")
    else:
        # Sharded: rank r steps worlds [r W, (r + 1) W) of an N W-world batch.
        n_all = args.worlds_per_rank * world_size
        sc = scenes.batched_worlds(n_worlds=n_all, worlds=multirank.shard(n_all, rank, world_size))
        w = GpuWorld.for_scene(sc, sc.params(), pairs_per_collider=6)
        workload = (f"batched worlds: {args.worlds_per_rank} worlds per GPU (of {n_all}), body counts "
                    f"log-uniform in [16, 2048] ({sc.num_dynamic} bodies on rank 0), ball piles and box stacks "
                    f"on their own grounds, dt 1/60, 8 velocity / 3 position iterations, one block per world")
    p = sc.params()
    stream = torch.cuda.ExternalStream(w.stream)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    n_dyn = sc.num_dynamic
    w.step(args.settle)
    # Launch shape chosen on real steps (every candidate gives the same bits).
    if args.schedule == "auto":
        tuned = w.autotune(5)
    else:
        tuned = ((1, 0) if args.schedule == "grid" else (2, args.world_threads)) + (0.0,)
        q = w.params
        q.solver_schedule, q.world_threads = tuned[0], tuned[1]
        w.set_params(q)
    p = w.params
    w.step(args.warmup)
    first_timed = int(w.counters()["steps"])

    # ---- device-resident timing -------------------------------------------------------
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world_size > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clocks:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xff)
            a, b = evs[k]
            a.record(stream)
            w.step(1, sync=False)
            b.record(stream)
        torch.cuda.synchronize()
        w.synchronize()
    if world_size > 1:
        torch.distributed.barrier()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = multirank.reduce_max(sum(step_ms), device="cuda")
    value = multirank.reduce_sum(n_dyn * args.steps, device="cuda") / (total_ms * 1e-3)

    # ---- end to end through the C ABI with host buffers ------------------------------------
    # Page-locked host arrays, as a host that streams every step would keep them.
    pos = pinned(np.zeros((len(sc.bodies), 7), np.float32))
    vel = pinned(np.zeros((len(sc.bodies), 6), np.float32))
    dyn = np.nonzero(sc.bodies["status"] == 2)[0]
    handles = pinned(np.ascontiguousarray(sc.body_handles[dyn]))
    forces = pinned(np.zeros((len(dyn), 6), np.float32))
    # One untimed pass first: it sizes the world's staging area for this batch.
    w.apply_forces(handles, forces, wake=False)
    w.step(1, sync=False)
    w.download_into(pos, vel)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        w.apply_forces(handles, forces, wake=False)
        w.step(1, sync=False)
        w.download_into(pos, vel)
    e2e_s = time.perf_counter() - t0
    h2d = handles.nbytes + forces.nbytes          # 16-byte handles and 6 force floats per dynamic body
    d2h = pos.nbytes + vel.nbytes                 # every body's pose and velocity
    e2e_value = multirank.reduce_sum(n_dyn * args.steps, device="cuda") / multirank.reduce_max(e2e_s, device="cuda")

    # ---- phase times (CUDA events on the world's stream), after the timed region ----------
    p.profile = 1
    w.set_params(p)
    counters = []
    for _ in range(PROFILE_STEPS):
        w.step(1)
        counters.append(w.counters())
    p.profile = 0
    w.set_params(p)

    # ---- roofline of the dominant kernel: the velocity solver (k_velocity) ------------------
    # Algorithmic bytes of one SOR-Prox iteration: 128 per solver contact
    # (normal, two lever arms, r / rhs / impulse of 3 rows, friction, 2 body
    # indices read; 3 impulses written) + 76 per dynamic body (Δv read and
    # written, inverse mass and inverse inertia read).
    peak, peak_kind = measured_peaks()
    K = statistics.mean(c["num_solver_contacts"] for c in counters)
    B = statistics.mean(c["num_active_bodies"] for c in counters)
    it = statistics.mean(c["velocity_iterations"] for c in counters)
    bytes_launch = it * (128 * K + 76 * B)
    solve_ms = statistics.mean(c["velocity_resolution_time"] for c in counters)
    achieved = bytes_launch / (solve_ms * 1e-3) / 1e9
    cl = clocks.summary()
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{workload}; timed steps "
                               f"{first_timed}..{first_timed + args.steps - 1} of the run",
                   "l2": "flushed (256 MiB write) between timed steps",
                   "solver_schedule": {1: "one cooperative grid",
                                       2: "per world: a cluster, a block or a warp each"}[tuned[0]],
                   "world_threads": tuned[1],
                   "parallelism": ("replicas" if args.workload in ("pile", "pyramid", "mixed")
                                   else f"worlds sharded over {world_size} GPUs"),
                   "contacts": int(statistics.mean(c["num_contacts"] for c in counters)),
                   "solver_contacts": int(K), "active_bodies": int(B),
                   "colours": int(statistics.mean(c["num_colours"] for c in counters))},
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "kernel": "k_velocity" if tuned[0] == 1 else "k_world_velocity", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": (VELOCITY_TRAFFIC_PER_LAUNCH if args.workload == "pile" and tuned[0] == 1
                                 else int(WORLD_VELOCITY_TRAFFIC_PER_CONTACT * K)
                                 if args.workload == "batched" and tuned[0] == 2 else None),
                     "peak_source": peak_kind,
                     "bytes_per_launch": bytes_launch, "launch_ms": solve_ms},
        "clocks": {"sm_mhz": cl["sm_mhz"], "sm_max_mhz": cl["sm_max_mhz"], "reasons": cl["reasons"]},
        "gpu_launches": (LAUNCHES_PER_STEP if tuned[0] == 1 else LAUNCHES_PER_STEP_BATCHED) * args.steps,
        "phase_ms": {k: statistics.mean(c[k] for c in counters) for k in
                     ("step_time", "solver_time", "collision_detection_time", "broad_phase_time", "narrow_phase_time",
                      "island_construction_time", "colouring_time", "assembly_time", "velocity_resolution_time",
                      "velocity_update_time", "position_resolution_time")},
    }
    if rank == 0 and world_size == 1 and args.workload == "pile" and not args.no_pgs_iterations:
        line["pgs_iterations"] = pgs_iterations(lambda: scenes.ball_pile(side=args.side), args.settle)
    if rank == 0 and world_size == 1 and not args.no_cpu_baseline and args.workload == "pile":
        line["cpu_baseline"] = cpu_baseline(lambda: scenes.ball_pile(side=args.side), args.cpu_seconds, args.settle)
    if rank == 0:
        print(json.dumps(line))
    if world_size > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

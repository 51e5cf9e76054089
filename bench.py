"""Benchmark of the GPU rigid-body step: body-steps/s and PGS iterations to 1e-4.

Headline workload (value, e2e, roofline): the 32^3 ball pile, 32768 balls of
radius 0.5 on a 1.2 lattice (seeded jitter), dropped on a static ground,
density 1, friction 0.3, dt 1/60, the reference's 8 velocity / 3 position
iterations. The pile is simulated untimed for --settle steps, then the
autotuner's steps, then --warmup steps, then --steps timed steps.

  value  body-steps/s with the world resident in HBM: CUDA events on the
         world's stream around each step, an L2 flush (256 MiB write)
         between steps, outside the timed region.
  e2e    the same metric through the C ABI as a host would drive it: per
         step, upload of the step's applied forces from pinned host memory,
         npgpu_step, download of every body's pose and velocity into host
         buffers; wall time of the loop.
  c4_batched  the batched-worlds record: 4096 worlds (body counts
         log-uniform in [16, 2048]) in one world object, timed the same way,
         roofline on the per-world velocity kernel.
  pgs_iterations  the metric's second half on the 100k mixed pile of balls
         and cuboids: SOR-Prox iterations to a residual of 1e-4 (cap 4096),
         impulse cache alone vs the learned warm start, whose network is
         trained in the run on 2M solver-converged contacts of this pile and
         of the 210-box pyramid.
  cpu_baseline  the CPU oracle (the restated reference step, f32, one
         thread) on the same pile and step window; cpu_configs adds the
         pyramid and a 10k-body subset of the mixed pile beside the GPU's
         own figure on the same steps.
  --impl reference  times the CPU oracle on this host instead (the Rust
         reference cannot be built here).
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
# Kernels of this library launched per step, from the ncu launch list of one
# step of this workload (every kernel is this library's: the broad phase's
# radix sort is 4 passes of 3 launches over 32-bit keys).
LAUNCHES_PER_STEP = 47
# The per-world schedule (6 sort passes over the batched worlds' 44-bit keys,
# the per-world bucketing, velocity, finish and position kernels), from the
# launch list of one step of a 1024-world batch.
LAUNCHES_PER_STEP_BATCHED = 65
# dram__bytes_read.sum + dram__bytes_write.sum of one k_velocity launch on this
# workload, from the ncu launch list of one step.
VELOCITY_TRAFFIC_PER_LAUNCH = 45570304 + 1165312
# dram__bytes_read.sum + dram__bytes_write.sum of one k_world_velocity launch
# on a 1024-world batch at step 63 (1 142 644 contacts, records larger than
# L2, so every sweep streams them), per contact: the batched line scales it by
# its own solver contacts.
WORLD_VELOCITY_TRAFFIC_PER_CONTACT = (1969872000 + 293148160) / 1142644


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
                    help="untimed steps first (default: 200 for the ball pile and the pyramid, 300 for the mixed "
                         "pile, 60 for batched worlds, 0 for the brick walls, whose impact phase is the workload)")
    ap.add_argument("--side", type=int, default=32)
    ap.add_argument("--workload", default="pile", choices=["pile", "batched", "pyramid", "walls", "mixed", "joints"],
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
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched-worlds record of the default (pile) run")
    ap.add_argument("--sweep-order", default="separate", choices=["separate", "manifold"],
                    help="velocity-solve row order: every friction row, then every normal row, each "
                         "iteration (separate: the reference's order), or each manifold's friction rows "
                         "then its normal rows in one sweep (manifold)")
    ap.add_argument("--ccd", action="store_true",
                    help="walls: the balls' colliders with continuous collision detection")
    args = ap.parse_args()
    if args.settle is None:
        args.settle = SETTLE[args.workload]
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


# Steps npgpu_autotune advances a single-world scene by: one automatic step,
# then 1 + 5 steps for each of its two candidates (the one grid, and the
# per-world schedule with the world on one thread-block cluster).
AUTOTUNE_STEPS_SINGLE_WORLD = 1 + 2 * (1 + 5)


def host_cpu():
    """Core count and model name of this host."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if model is None:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
            for line in out.splitlines():
                if line.lower().startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return os.cpu_count(), model


def cpu_sample(scene, first_step, max_steps, seconds, what):
    """Times the oracle (the restated reference step, f32, one thread, the
    reference's row order) on a bounded sample of a workload: the scene is
    stepped `first_step` untimed steps, then up to `max_steps` steps are timed,
    stopping after about `seconds`."""
    from oracle.oracle_py import ORDER_REFERENCE, OracleWorld
    o = OracleWorld(scene.params(), scene.gravity, precision=32, order=ORDER_REFERENCE)
    o.load_scene(scene)
    o.step(first_step)
    steps = 0
    t0 = time.perf_counter()
    while steps < max_steps and (steps == 0 or time.perf_counter() - t0 < seconds):
        o.step(1)
        steps += 1
    dt = time.perf_counter() - t0
    c = o.counters()
    o.close()
    sample = (f"steps {first_step}..{first_step + steps - 1} of {what} ({c['num_contacts']} contacts at the "
              "end), single-threaded f32 oracle in the reference's row order, built -O3; the Rust reference "
              "has no toolchain on this host")
    return scene.num_dynamic * steps / dt, steps, dt, sample


def cpu_baseline_line(value, sample):
    cores, model = host_cpu()
    return {"value": value, "unit": METRIC, "cores": 1, "host_cores": cores, "cpu_model": model, "kind": "port",
            "sample": sample}


def pile_window(args):
    """First timed step of the ball-pile workload on the GPU arm: the settle
    steps, the autotuner's steps, then the warm-up steps."""
    return args.settle + AUTOTUNE_STEPS_SINGLE_WORLD + args.warmup


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from nphysics_gb300 import scenes
    n_dyn = args.side ** 3
    first = pile_window(args)
    value, steps, dt, sample = cpu_sample(scenes.ball_pile(side=args.side), first, args.steps,
                                          max(5.0, args.cpu_seconds), f"the {n_dyn}-ball pile")
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"ball pile {args.side}^3 = {n_dyn} balls (radius 0.5, 1.2 lattice, seeded jitter) "
                               f"on a static ground, dt 1/60, 8 velocity / 3 position iterations; timed steps "
                               f"{first}..{first + steps - 1} of the run (the GPU arm's window starts at the "
                               "same step)",
                   "sample": sample},
        "cpu_baseline": cpu_baseline_line(value, sample),
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def _iteration_stats(its, cap):
    s = sorted(its)
    return {"iterations_mean": statistics.mean(its), "iterations_p95": s[min(len(s) - 1, int(0.95 * len(s)))],
            "iterations_max": s[-1], "steps_at_cap": sum(1 for i in its if i >= cap)}


def _record_steps(w, steps, tolerance, max_iterations, capacity):
    """Samples (features, converged impulses) of every solver contact of the
    next `steps` steps of `w`, each solved to `tolerance`."""
    import numpy as np
    saved = w.params
    p = w.params
    p.solve_to_tolerance = 1
    p.residual_tolerance = tolerance
    p.max_iterations_to_tolerance = max_iterations
    w.set_params(p)
    out = []
    for _ in range(steps):
        w.mlp_record(capacity)
        w.step(1)
        out.append(w.mlp_samples())
        w.mlp_record(0)
    p.solve_to_tolerance = 0
    w.set_params(p)
    return np.concatenate(out) if out else np.zeros((0, 28), np.float32)


def pgs_iterations(mixed, settle=300, steps=20, cap=4096, samples_total=2_000_000, train_steps=4000):
    """The metric's second half on the 100k mixed pile (C3): SOR-Prox
    iterations to a residual of 1e-4 (at most `cap`) with the impulse cache
    alone and with the learned warm start, over `steps` steps after `settle`
    steps with the default parameters (both worlds reach the comparison with
    the same bits).

    Training set: 2M solver-converged contacts (each step solved to 1e-5),
    80 % from the mixed pile (one step in 30 of its settle, from step 60 on)
    and 20 % from the 210-box pyramid (its first 300 steps), drawn by a seeded
    subsample; the network trains on the GPU with Adam (lr 1e-3, batch 4096)."""
    import numpy as np

    from nphysics_gb300 import abi, scenes
    from nphysics_gb300.world import GpuWorld
    t0 = time.perf_counter()
    rng = np.random.default_rng(2024)
    rec = GpuWorld.for_scene(mixed, mixed.params(), pairs_per_collider=12)
    parts = []
    done = 0
    for mark in range(60, settle + 1, 30):
        rec.step(mark - done)
        parts.append(_record_steps(rec, 1, 1e-5, 1024, 4_000_000))
        done = mark + 1
    c3 = np.concatenate(parts)
    pyr = GpuWorld.for_scene(scenes.pyramid(base=20))
    c1 = _record_steps(pyr, 300, 1e-5, 1024, 4_000_000)
    pyr.close()
    n3 = min(len(c3), int(0.8 * samples_total))
    n1 = min(len(c1), samples_total - n3)
    data = np.concatenate([c3[rng.choice(len(c3), n3, replace=False)], c1[rng.choice(len(c1), n1, replace=False)]])
    rec.mlp_load_samples(data)
    rec.mlp_train(1, batch=4096, lr=1e-3, seed=1, init=True)
    loss = rec.mlp_train(train_steps, batch=4096, lr=1e-3, seed=2)
    net = rec.mlp_get()
    rec.close()
    t_train = time.perf_counter() - t0
    out = {"scene": "mixed pile, 100000 balls and cuboids dropped from U(1, 60) over 100 x 100",
           "tolerance": 1e-4, "max_iterations": cap, "steps": f"{settle}..{settle + steps - 1}",
           "network": f"trained in this run: {len(data)} samples ({n3} from the mixed pile, {n1} from the "
                      f"210-box pyramid), solved to 1e-5, {train_steps} Adam steps (batch 4096, lr 1e-3), "
                      f"final loss {loss:.3f}, {t_train:.1f} s"}
    # The third arm keeps the plain start and solves each manifold's friction
    # rows and then its normal rows in one sweep (the same rows, another
    # Gauss-Seidel order), for its convergence per iteration beside the
    # reference's order.
    for name, mode, sweep in (("plain", abi.WARMSTART_CACHE, abi.SWEEP_SEPARATE),
                              ("learned", abi.WARMSTART_LEARNED, abi.SWEEP_SEPARATE),
                              ("plain_per_manifold_order", abi.WARMSTART_CACHE, abi.SWEEP_MANIFOLD)):
        w = GpuWorld.for_scene(mixed, mixed.params(), pairs_per_collider=12)
        w.mlp_set(net)
        w.step(settle)
        p = w.params
        p.warmstart_mode = mode
        p.sweep_order = sweep
        p.solve_to_tolerance = 1
        p.residual_tolerance = 1e-4
        p.max_iterations_to_tolerance = cap
        w.set_params(p)
        its, r0, ms, starts, kept, contacts = [], [], [], 0, 0, []
        for _ in range(steps):
            a = time.perf_counter()
            w.step(1)
            ms.append(time.perf_counter() - a)
            c = w.counters()
            its.append(c["velocity_iterations"])
            r0.append(c["residual_initial"])
            starts += c["learned_starts"]
            kept += c["learned_kept"]
            contacts.append(c["num_solver_contacts"])
        out[name] = dict(_iteration_stats(its, cap), residual_after_warm_start=statistics.mean(r0),
                         body_steps_per_s=mixed.num_dynamic * steps / sum(ms),
                         solver_contacts_mean=statistics.mean(contacts))
        if mode == abi.WARMSTART_LEARNED:
            out[name]["learned_starts"] = starts
            out[name]["learned_kept"] = kept
        w.close()
    out["iterations_ratio_plain_over_learned"] = out["plain"]["iterations_mean"] / out["learned"]["iterations_mean"]
    out["body_steps_ratio_learned_over_plain"] = (out["learned"]["body_steps_per_s"] /
                                                  out["plain"]["body_steps_per_s"])
    out["iterations_ratio_plain_over_per_manifold_order"] = (out["plain"]["iterations_mean"] /
                                                             out["plain_per_manifold_order"]["iterations_mean"])
    out["seconds"] = time.perf_counter() - t0
    return out


def walls_record(steps=240, settle=30, tol_steps=20, cap=4096):
    """BASELINE's C5 report on a two-wall subset (each wall 50 x 40 bricks and
    64 balls, the bench's recipe): the GPU's maximum penetration, kinetic
    energy and contacts beside the f64 oracle's (the reference's order) over
    `steps` steps, and iterations to 1e-4 with the impulse cache alone and
    with the learned start trained on the subset's own solver-converged
    contacts (steps settle..settle + tol_steps - 1)."""
    import numpy as np

    from nphysics_gb300 import abi, scenes
    from nphysics_gb300.world import GpuWorld
    from oracle.oracle_py import ORDER_REFERENCE, OracleWorld
    t0 = time.perf_counter()
    sc = scenes.brick_walls(n_walls=2, seed=1234)
    g = GpuWorld.for_scene(sc, sc.params(), pairs_per_collider=8)
    r = OracleWorld(sc.params(), sc.gravity, precision=64, order=ORDER_REFERENCE)
    r.load_scene(sc)
    ke_g, ke_r, pen_g, pen_r = [], [], [], []
    for _ in range(steps):
        g.step(1)
        r.step(1)
        cg, cr = g.counters(), r.counters()
        ke_g.append(cg["kinetic_energy"])
        ke_r.append(cr["kinetic_energy"])
        pen_g.append(cg["max_penetration"])
        pen_r.append(cr["max_penetration"])
    g.close()
    ke_g, ke_r = np.array(ke_g), np.array(ke_r)
    out = {"scene": "2 brick walls (50 x 40 bricks, 64 balls each), dt 1/120", "steps": steps,
           "max_penetration_gpu": max(pen_g), "max_penetration_f64": max(pen_r),
           "kinetic_energy_drift_vs_f64": float(np.max(np.abs(ke_g - ke_r)) / ke_r[0]),
           "kinetic_energy_initial": float(ke_r[0]), "kinetic_energy_final_gpu": float(ke_g[-1]),
           "kinetic_energy_final_f64": float(ke_r[-1]), "contacts_final_gpu": cg["num_contacts"],
           "contacts_final_f64": cr["num_contacts"]}
    rec = GpuWorld.for_scene(sc, sc.params(), pairs_per_collider=8)
    p = rec.params
    p.solve_to_tolerance, p.residual_tolerance, p.max_iterations_to_tolerance = 1, 1e-5, 1024
    rec.set_params(p)
    rec.mlp_record(4_000_000)
    rec.step(settle + tol_steps)
    rec.mlp_record(0)
    rec.mlp_train(1, batch=4096, lr=1e-3, seed=1, init=True)
    rec.mlp_train(3000, batch=4096, lr=1e-3, seed=2)
    net = rec.mlp_get()
    rec.close()
    for name, mode in (("plain", abi.WARMSTART_CACHE), ("learned", abi.WARMSTART_LEARNED)):
        w = GpuWorld.for_scene(sc, sc.params(), pairs_per_collider=8)
        w.mlp_set(net)
        w.step(settle)
        q = w.params
        q.warmstart_mode, q.solve_to_tolerance = mode, 1
        q.residual_tolerance, q.max_iterations_to_tolerance = 1e-4, cap
        w.set_params(q)
        its = []
        for _ in range(tol_steps):
            w.step(1)
            its.append(w.counters()["velocity_iterations"])
        out["iterations_to_1e-4_" + name] = _iteration_stats(its, cap)
        w.close()
    out["seconds"] = time.perf_counter() - t0
    return out


def gpu_window_rate(scene, first, steps, **kw):
    """Body-steps/s of the GPU step over steps first..first+steps-1 of the
    scene (CUDA events on the world's stream around the window), with the
    launch shape the autotuner picks for it on a separate copy of the world."""
    import torch

    from nphysics_gb300.world import GpuWorld
    probe = GpuWorld.for_scene(scene, scene.params(), **kw)
    probe.step(first)
    schedule, threads, _ = probe.autotune(3)
    probe.close()
    p = scene.params()
    p.solver_schedule, p.world_threads = schedule, threads
    w = GpuWorld.for_scene(scene, p, **kw)
    w.step(first)
    stream = torch.cuda.ExternalStream(w.stream)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    w.step(steps, sync=False)
    b.record(stream)
    w.synchronize()
    torch.cuda.synchronize()
    w.close()
    return scene.num_dynamic * steps / (a.elapsed_time(b) * 1e-3)


def cpu_configs(seconds):
    """The oracle beside the GPU on the pyramid and a 10k-body subset of the
    mixed pile, each on the same step window on both sides."""
    from nphysics_gb300 import scenes
    out = []
    for name, scene, first, steps, kw in (
            ("C1 box pyramid, 210 cuboids", scenes.pyramid(base=20), 5, 200, {}),
            ("C3 subset: 10000 balls and cuboids at the mixed pile's density (footprint 31.6 x 31.6, heights "
             "U(1, 60))", scenes.mixed_pile(n=10_000, footprint=31.6), 5, 120, {"pairs_per_collider": 12})):
        cpu, n, dt, sample = cpu_sample(scene, first, steps, seconds, name)
        gpu = gpu_window_rate(scene, first, n, **kw)
        out.append({"config": name, "steps": f"{first}..{first + n - 1}", "cpu_body_steps_per_s": cpu,
                    "gpu_body_steps_per_s": gpu, "sample": sample})
    return out


def whole_job(units_per_rank, device_ms, e2e_s, device="cuda"):
    """The whole job's value and e2e of a run on every rank: the units all
    ranks processed over the slowest rank's device time and end-to-end time
    (one process: its own figures)."""
    from nphysics_gb300 import multirank
    total_ms = multirank.reduce_max(device_ms, device)
    units = multirank.reduce_sum(units_per_rank, device)
    return units / (total_ms * 1e-3), units / multirank.reduce_max(e2e_s, device), total_ms


def measure(args, sc, w, kind, rank, world_size, local_rank):
    """Device-resident and end-to-end body-steps/s of world `w` on scene `sc`,
    plus the phase times and the velocity solver's roofline."""
    import numpy as np
    import torch

    stream = torch.cuda.ExternalStream(w.stream)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    n_dyn = sc.num_dynamic
    w.step(args.settle if kind == args.workload else SETTLE[kind])
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
    value, e2e_value, total_ms = whole_job(n_dyn * args.steps, sum(step_ms), e2e_s)

    # ---- phase times (CUDA events on the world's stream), after the timed region ----------
    p.profile = 1
    w.set_params(p)
    counters = []
    for _ in range(PROFILE_STEPS):
        w.step(1)
        counters.append(w.counters())
    p.profile = 0
    w.set_params(p)

    # ---- roofline of the dominant kernel: the velocity solver -------------------------------
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
    launches = LAUNCHES_PER_STEP if tuned[0] == 1 else LAUNCHES_PER_STEP_BATCHED
    if getattr(args, "ccd", False) and kind == "walls":
        # k_ccd_begin, the pair adjacency's count, scan (3), fill and sort,
        # k_ccd_world and k_ccd_solve once a pass (max_ccd_substeps + 2
        # passes), k_ccd_finish.
        launches += 8 + 2 * (int(p.max_ccd_substeps) + 2)
    return {
        "value": value, "ms_per_step": total_ms / args.steps, "first_timed_step": first_timed,
        "tuned": tuned,
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "kernel": "k_velocity" if tuned[0] == 1 else "k_world_velocity",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (VELOCITY_TRAFFIC_PER_LAUNCH if kind == "pile" and tuned[0] == 1
                                 else int(WORLD_VELOCITY_TRAFFIC_PER_CONTACT * K)
                                 if kind == "batched" and tuned[0] == 2 else None),
                     "peak_source": peak_kind, "bytes_per_launch": bytes_launch, "launch_ms": solve_ms},
        "clocks": {"sm_mhz": cl["sm_mhz"], "sm_max_mhz": cl["sm_max_mhz"], "reasons": cl["reasons"]},
        "gpu_launches": launches * args.steps,
        "counters": {"contacts": int(statistics.mean(c["num_contacts"] for c in counters)),
                     "solver_contacts": int(K), "active_bodies": int(B),
                     "colours": int(statistics.mean(c["num_colours"] for c in counters)),
                     "ccd_substeps": statistics.mean(c["ccd_substeps"] for c in counters),
                     "ccd_impacts": statistics.mean(c["ccd_impacts"] for c in counters)},
        "phase_ms": {k: statistics.mean(c[k] for c in counters) for k in
                     ("step_time", "solver_time", "collision_detection_time", "broad_phase_time", "narrow_phase_time",
                      "island_construction_time", "colouring_time", "assembly_time", "velocity_resolution_time",
                      "velocity_update_time", "position_resolution_time", "ccd_toi_computation_time",
                      "ccd_solver_time", "ccd_broad_phase_time", "ccd_narrow_phase_time", "ccd_world_time_max")},
    }


SETTLE = {"pile": 200, "batched": 60, "pyramid": 200, "walls": 0, "mixed": 300, "joints": 60}


def _params(sc, args):
    from nphysics_gb300 import abi
    p = sc.params()
    p.sweep_order = abi.SWEEP_MANIFOLD if args.sweep_order == "manifold" else abi.SWEEP_SEPARATE
    return p


def build_workload(kind, args, rank, world_size):
    from nphysics_gb300 import multirank, scenes
    from nphysics_gb300.world import GpuWorld
    if kind == "pile":
        # Replicas: every rank runs its own copy of the pile (one world per GPU).
        sc = scenes.ball_pile(side=args.side)
        w = GpuWorld.for_scene(sc, _params(sc, args))
        desc = (f"ball pile {args.side}^3 = {sc.num_dynamic} balls (radius 0.5, 1.2 lattice, seeded jitter) "
                f"on a static ground, dt 1/60, 8 velocity / 3 position iterations")
    elif kind == "pyramid":
        sc = scenes.pyramid(base=20)
        w = GpuWorld.for_scene(sc, _params(sc, args))
        desc = ("box pyramid: 210 cuboids of half extent 0.5 in a 20-base triangle on a static ground, "
                "density 1, friction 0.5, dt 1/60, 8 velocity / 3 position iterations")
    elif kind == "mixed":
        # Replicas: the 100k mixed pile of balls and cuboids on every rank.
        sc = scenes.mixed_pile(n=100_000)
        w = GpuWorld.for_scene(sc, _params(sc, args), pairs_per_collider=12)
        desc = ("mixed pile: 100000 bodies, half balls of radius U(0.2, 0.8), half cuboids of half extents "
                "U(0.2, 0.8)^3 at uniform random orientations, density 1, friction 0.5, dropped from heights "
                "U(1, 60) over a 100 x 100 footprint onto a static ground, dt 1/60, 8 velocity / 3 position "
                "iterations")
    elif kind == "walls":
        # Each rank steps its own 256 walls (weak scaling).
        sc = scenes.brick_walls(n_walls=256, seed=1234 + rank, ccd=args.ccd)
        w = GpuWorld.for_scene(sc, _params(sc, args), pairs_per_collider=8)
        desc = ("brick walls: 256 walls per GPU of 50 x 40 bricks (half extents 0.5 x 0.25 x 0.25, running "
                "bond), each struck by 64 balls of radius 0.4, density 10, at U(20, 40) m/s; friction 0.6, "
                "dt 1/120, 8 velocity / 3 position iterations" +
                ("; the balls' colliders with CCD (one substep a step at most)" if args.ccd else ""))
    elif kind == "joints":
        # Sharded like the batched worlds: worlds of every joint kind with contacts.
        n_all = args.worlds_per_rank * world_size
        sc = scenes.batched_zoo(n_worlds=n_all, worlds=multirank.shard(n_all, rank, world_size))
        w = GpuWorld.for_scene(sc, _params(sc, args))
        desc = (f"jointed worlds: {args.worlds_per_rank} worlds per GPU (of {n_all}), each a ground with one joint of "
                f"each of the ten kinds (ball, fixed, revolute, cartesian, planar, rectangular, universal, prismatic "
                f"with offset limits, cylindrical, pin-slot) on boxes and balls and free boxes falling on them "
                f"({sc.num_dynamic} bodies, {len(sc.joints)} joints on rank 0), dt 1/60, 8 velocity / 3 position "
                f"iterations")
    else:
        # Sharded: rank r steps worlds [r W, (r + 1) W) of an N W-world batch.
        n_all = args.worlds_per_rank * world_size
        sc = scenes.batched_worlds(n_worlds=n_all, worlds=multirank.shard(n_all, rank, world_size))
        w = GpuWorld.for_scene(sc, _params(sc, args), pairs_per_collider=6)
        desc = (f"batched worlds: {args.worlds_per_rank} worlds per GPU (of {n_all}), body counts "
                f"log-uniform in [16, 2048] ({sc.num_dynamic} bodies on rank 0), ball piles and box stacks "
                f"on their own grounds, dt 1/60, 8 velocity / 3 position iterations, one block per world")
    return sc, w, desc


def run_gpu(args):
    import torch

    from nphysics_gb300 import build, multirank, scenes

    rank, world_size, local_rank = multirank.rank_env()
    torch.cuda.set_device(local_rank)
    if world_size > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build.build()
    torch.cuda.init()
    sc, w, desc = build_workload(args.workload, args, rank, world_size)
    m = measure(args, sc, w, args.workload, rank, world_size, local_rank)
    w.close()
    tuned = m["tuned"]
    line = {
        "metric": METRIC, "value": m["value"], "unit": METRIC, "n_gpus": world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": m["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict({"workload": f"{desc}; timed steps {m['first_timed_step']}..."
                                    f"{m['first_timed_step'] + args.steps - 1} of the run",
                        "l2": "flushed (256 MiB write) between timed steps",
                        "solver_schedule": {1: "one cooperative grid",
                                            2: "per world: a cluster, a block or a warp each"}[tuned[0]],
                        "world_threads": tuned[1],
                        "sweep_order": {"separate": "every friction row, then every normal row (the reference's)",
                                        "manifold": "each manifold's friction rows, then its normal rows"}[
                                            args.sweep_order],
                        "parallelism": ("replicas" if args.workload in ("pile", "pyramid", "mixed")
                                        else f"worlds sharded over {world_size} GPUs")}, **m["counters"]),
        "e2e": m["e2e"], "roofline": m["roofline"], "clocks": m["clocks"], "gpu_launches": m["gpu_launches"],
        "phase_ms": m["phase_ms"],
    }
    if args.workload == "pile" and m["first_timed_step"] != pile_window(args):
        line["config"]["window_note"] = (f"the reference arm's window starts at step {pile_window(args)}, this "
                                         f"arm's at {m['first_timed_step']}")
    if args.workload == "pile" and not args.no_batched:
        # The batched-worlds record (C4), measured the same way on this GPU.
        bsc, bw, bdesc = build_workload("batched", args, rank, world_size)
        bm = measure(args, bsc, bw, "batched", rank, world_size, local_rank)
        bw.close()
        line["c4_batched"] = {"workload": bdesc, "value": bm["value"], "unit": METRIC,
                              "ms_per_step": bm["ms_per_step"], "e2e": bm["e2e"], "roofline": bm["roofline"],
                              "clocks": bm["clocks"], "gpu_launches": bm["gpu_launches"], "phase_ms": bm["phase_ms"],
                              "timed_steps": f"{bm['first_timed_step']}..{bm['first_timed_step'] + args.steps - 1}",
                              "world_threads": bm["tuned"][1], **bm["counters"]}
    if rank == 0 and world_size == 1 and args.workload == "walls" and not args.ccd:
        line["c5_report"] = walls_record()
    if rank == 0 and world_size == 1 and args.workload == "pile" and not args.no_pgs_iterations:
        line["pgs_iterations"] = pgs_iterations(scenes.mixed_pile(n=100_000))
    if rank == 0 and world_size == 1 and not args.no_cpu_baseline and args.workload == "pile":
        first = m["first_timed_step"]
        value, steps, dt, sample = cpu_sample(scenes.ball_pile(side=args.side), first, 10 ** 9, args.cpu_seconds,
                                              f"the same {sc.num_dynamic}-ball pile")
        line["cpu_baseline"] = cpu_baseline_line(value, sample)
        line["cpu_configs"] = cpu_configs(args.cpu_seconds)
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

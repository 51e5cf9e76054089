"""The learned warm start: the network's gradient against the CPU
restatement, the fused inference against the oracle, training, and what the
trained network gains over the impulse cache alone.

Tolerances: gradients within 2e-3 relative (fp32 sums of 64-sample tiles
added atomically on the GPU against float64 on the CPU); the learned step is
bitwise equal to the oracle's colour order (same features, same bf16-weight
forward pass, same residual check)."""
import numpy as np
import pytest

from nphysics_gb300 import abi, scenes
from oracle import mlp_ref
from oracle.oracle_py import ORDER_COLOUR, OracleWorld


def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    s = rng.normal(size=(40, abi.MLP_SAMPLE_FLOATS)).astype(np.float32)
    p = mlp_ref.random_params(rng, s)
    _, g = mlp_ref.loss_and_grad(p, s)
    eps = 1e-3
    for i in (mlp_ref.B2 + 10, mlp_ref.B3, mlp_ref.B3 + 1, mlp_ref.B3 + 2):
        q = p.copy()
        q[i] += eps
        lp, _ = mlp_ref.loss_and_grad(q, s)
        q[i] -= 2 * eps
        lm, _ = mlp_ref.loss_and_grad(q, s)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 2e-2 * abs(g[i]) + 1e-5, (i, fd, g[i])


def test_oracle_learned_start_runs():
    # The oracle's learned warm start on a small pile: it runs and stays finite.
    sc = scenes.random_cluster(n=20, seed=2)
    p = sc.params()
    p.warmstart_mode = abi.WARMSTART_LEARNED
    o = OracleWorld(p, sc.gravity, precision=32, order=ORDER_COLOUR)
    o.load_scene(sc)
    o.mlp_set(mlp_ref.random_params(np.random.default_rng(1)))
    o.step(20)
    assert np.isfinite(o.bodies()["position"]).all()


@pytest.mark.gpu
def test_gradient_matches_reference(gpu_lib):
    from nphysics_gb300.world import GpuWorld
    rng = np.random.default_rng(3)
    s = rng.normal(size=(300, abi.MLP_SAMPLE_FLOATS)).astype(np.float32)
    s[:, :24] *= rng.uniform(0.1, 10.0, size=24).astype(np.float32)
    p = mlp_ref.random_params(rng, s)
    sc = scenes.random_cluster(n=4, seed=1)
    g = GpuWorld.for_scene(sc)
    g.mlp_set(p)
    grad, loss = g.mlp_grad(s)
    rloss, rgrad = mlp_ref.loss_and_grad(p, s)
    assert abs(loss - rloss) <= 1e-5 * abs(rloss) + 1e-6
    err = np.abs(grad - rgrad)
    assert (err <= 2e-3 * np.abs(rgrad) + 2e-3 * np.abs(rgrad).max()).all(), err.max()
    np.testing.assert_array_equal(g.mlp_get(), p)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [abi.WARMSTART_LEARNED, abi.WARMSTART_LEARNED_ALL])
@pytest.mark.parametrize("schedule", [abi.SCHEDULE_GRID, abi.SCHEDULE_WORLDS])
def test_learned_step_matches_oracle(gpu_lib, schedule, mode):
    # Mode 2 starts new contacts from the network, mode 3 every contact; each
    # prediction is checked against the start it replaces.
    from nphysics_gb300.world import GpuWorld
    sc = scenes.random_cluster(n=30, seed=6)
    if schedule == abi.SCHEDULE_WORLDS:
        sc = scenes.batched_worlds(n_worlds=4, seed=5, lo=8, hi=40)
    p = sc.params()
    p.warmstart_mode = mode
    p.solver_schedule = schedule
    net = mlp_ref.random_params(np.random.default_rng(7))
    net[mlp_ref.YS:mlp_ref.PARAMS] = 0.05     # predictions of a plausible impulse size
    g = GpuWorld.for_scene(sc, p)
    g.mlp_set(net)
    o = OracleWorld(p, sc.gravity, precision=32, order=ORDER_COLOUR)
    o.load_scene(sc)
    o.mlp_set(net)
    g.step(25)
    o.step(25)
    np.testing.assert_array_equal(g.bodies()["position"], o.bodies()["position"])
    np.testing.assert_array_equal(g.bodies()["velocity"], o.bodies()["velocity"])


@pytest.mark.gpu
def test_learned_mode_needs_a_network(gpu_lib):
    from nphysics_gb300.world import GpuWorld, NpgpuError
    sc = scenes.random_cluster(n=4, seed=1)
    p = sc.params()
    p.warmstart_mode = abi.WARMSTART_LEARNED
    g = GpuWorld.for_scene(sc, p)
    with pytest.raises(NpgpuError, match="INVALID_ARGUMENT"):
        g.step(1)


def _record(scene, steps, capacity=400_000):
    """Runs `steps` steps solved to a residual of 1e-5 while recording samples."""
    from nphysics_gb300.world import GpuWorld
    p = scene.params()
    p.solve_to_tolerance = 1
    p.residual_tolerance = 1e-5
    p.max_iterations_to_tolerance = 200
    g = GpuWorld.for_scene(scene, p)
    g.mlp_record(capacity)
    g.step(steps)
    g.mlp_record(0)
    return g


@pytest.mark.gpu
def test_training_reduces_loss(gpu_lib):
    g = _record(scenes.ball_pile(side=8), steps=60)
    s = g.mlp_samples()
    assert len(s) > 5000
    assert np.isfinite(s).all()
    first = g.mlp_train(1, batch=1024, lr=1e-3, seed=3, init=True)
    last = g.mlp_train(400, batch=1024, lr=1e-3, seed=4)
    assert last < 0.5 * first, (first, last)


@pytest.mark.gpu
def test_trained_network_lowers_the_warm_start_residual(gpu_lib):
    # Train on the solver's own converged impulses of a 1000-ball pile, then
    # run the pile again with and without the network (8 iterations a step):
    # the residual after the warm start, averaged over the steps with
    # contacts, drops (measured: about 30% on a 4096-ball pile).
    from nphysics_gb300.world import GpuWorld
    sc = scenes.ball_pile(side=10)
    g = _record(sc, steps=150)
    g.mlp_train(1, batch=4096, lr=1e-3, seed=1, init=True)
    g.mlp_train(1500, batch=4096, lr=1e-3, seed=2)
    net = g.mlp_get()
    out = {}
    for mode in (abi.WARMSTART_CACHE, abi.WARMSTART_LEARNED):
        p = sc.params()
        p.warmstart_mode = mode
        w = GpuWorld.for_scene(sc, p)
        if mode == abi.WARMSTART_LEARNED:
            w.mlp_set(net)
        r0, kept = [], 0
        for _ in range(150):
            w.step(1)
            c = w.counters()
            if c["num_solver_contacts"]:
                r0.append(c["residual_initial"])
            kept += c["learned_kept"]
        out[mode] = (float(np.mean(r0)), kept)
    plain, learned = out[abi.WARMSTART_CACHE], out[abi.WARMSTART_LEARNED]
    assert learned[1] > 0
    assert learned[0] < 0.9 * plain[0], (plain, learned)

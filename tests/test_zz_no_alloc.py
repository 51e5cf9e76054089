"""npgpu_find_pairs_static: the broad phase for callers that cannot allocate.

Callers that cannot call cudaMalloc (real-time loops that must not block on
the allocator, plugins whose host application owns all device memory) get
the broad phase over device buffers they already own, with all scratch in a
fixed array inside the library. Its pairs must equal the world's own broad
phase (npgpu_get_pairs) on the same fat AABBs, call after call, and a
brute-force host check on the edge cases: no box, one, two, identical boxes,
a pair buffer smaller than the pair count, and group ids above 16 bits.
"""
import ctypes as C

import numpy as np
import pytest

from nphysics_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _call(lib, aabbs, groups, max_pairs):
    """One call through the C ABI; returns (reported count, written pairs)."""
    import torch
    aabbs = np.ascontiguousarray(aabbs, np.float32).reshape(-1, 6)
    d_aabb = torch.from_numpy(aabbs).cuda() if len(aabbs) else None
    d_groups = (torch.from_numpy(np.ascontiguousarray(groups, np.uint32).view(np.int32)).cuda()
                if groups is not None else None)
    d_pairs = torch.full((max(max_pairs, 1), 2), -1, dtype=torch.int32, device="cuda")
    d_count = torch.full((1,), 12345, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = lib.npgpu_find_pairs_static(C.c_void_p(d_aabb.data_ptr()) if d_aabb is not None else None,
                                     C.c_void_p(d_groups.data_ptr()) if d_groups is not None else None,
                                     len(aabbs), C.c_void_p(d_pairs.data_ptr()), max_pairs,
                                     C.c_void_p(d_count.data_ptr()), None)
    assert st == abi.OK, lib.npgpu_last_error(None)
    torch.cuda.synchronize()
    n = int(d_count.cpu().numpy().view(np.uint32)[0])
    assert n != 0xffffffff
    written = d_pairs[:min(n, max_pairs)].cpu().numpy().view(np.uint32)
    return n, written


def _sorted(p):
    p = np.asarray(p, np.uint32).reshape(-1, 2)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


def _static_pairs(lib, aabbs, groups, max_pairs):
    n, p = _call(lib, aabbs, groups, max_pairs)
    assert n <= max_pairs
    return _sorted(p)


def _brute_force(aabbs, groups=None):
    """Pairs (i < j) of closed boxes that intersect, within one group."""
    a = np.asarray(aabbs, np.float32).reshape(-1, 6)
    i, j = np.triu_indices(len(a), 1)
    hit = np.all((a[i, :3] <= a[j, 3:]) & (a[j, :3] <= a[i, 3:]), axis=1)
    if groups is not None:
        g = np.asarray(groups, np.uint32)
        hit &= g[i] == g[j]
    return _sorted(np.stack([i[hit], j[hit]], axis=1))


def test_static_pairs_match_the_world_broad_phase(gpu_lib):
    from nphysics_gb300.world import GpuWorld
    lib = gpu_lib
    sc = scenes.random_cluster(n=600, seed=21, extent=6.0)
    w = GpuWorld.for_scene(sc)
    w.step(2)
    want = w.pairs()
    aabbs = w.aabbs()
    assert len(want) > 300
    for _ in range(2):   # two calls in a row share the scratch array
        got = _static_pairs(lib, aabbs, None, 16 * len(aabbs))
        np.testing.assert_array_equal(got, want)


def test_static_pairs_respect_groups(gpu_lib):
    from nphysics_gb300.world import GpuWorld
    lib = gpu_lib
    one = scenes.random_cluster(n=200, seed=8, extent=3.0)
    two_b = np.concatenate([one.bodies, one.bodies.copy()])
    two_b["world"][len(one.bodies):] = 1
    two_c = np.concatenate([one.colliders, one.colliders.copy()])
    two_c["body"]["index"][len(one.colliders):] += len(one.bodies)
    sc = scenes.Scene("two worlds", two_b, two_c)
    w = GpuWorld.for_scene(sc)
    w.step(1)
    want = w.pairs()
    groups = sc.bodies["world"][sc.colliders["body"]["index"]].astype(np.int32)
    for _ in range(2):
        got = _static_pairs(lib, w.aabbs(), groups, 16 * len(groups))
        np.testing.assert_array_equal(got, want)


def test_static_pairs_reject_too_many_boxes(gpu_lib):
    lib = gpu_lib
    cnt = (C.c_uint32 * 1)()
    st = lib.npgpu_find_pairs_static(C.c_void_p(1), None, 32769, None, 0, cnt, None)
    assert st == abi.ERR_CAPACITY
    assert b"32768" in lib.npgpu_last_error(None)


def test_static_pairs_small_and_degenerate_inputs(gpu_lib):
    lib = gpu_lib
    box = [0.0, 0.0, 0.0, 1.0, 1.0, 1.0]
    # No box, one box: no pair, count 0.
    assert _call(lib, np.zeros((0, 6)), None, 4)[0] == 0
    assert _call(lib, [box], None, 4)[0] == 0
    # Two boxes: touching faces count (closed boxes), apart does not.
    assert _static_pairs(lib, [box, [1.0, 0.0, 0.0, 2.0, 1.0, 1.0]], None, 4).tolist() == [[0, 1]]
    assert _call(lib, [box, [1.5, 0.0, 0.0, 2.0, 1.0, 1.0]], None, 4)[0] == 0
    # Identical boxes (identical sort keys): every pair, once.
    same = np.tile(np.float32(box), (40, 1))
    for _ in range(2):
        np.testing.assert_array_equal(_static_pairs(lib, same, None, 40 * 39 // 2), _brute_force(same))


def test_static_pairs_truncate_to_the_buffer(gpu_lib):
    # More pairs than slots: *count holds the full total, only max_pairs pairs
    # are written, and each written pair is a true pair.
    lib = gpu_lib
    rng = np.random.default_rng(3)
    lo = rng.uniform(0, 4, (300, 3)).astype(np.float32)
    aabbs = np.concatenate([lo, lo + rng.uniform(0.3, 1.0, (300, 3)).astype(np.float32)], axis=1)
    want = _brute_force(aabbs)
    assert len(want) > 200
    for max_pairs in (0, 1, 57, len(want) - 1):
        n, written = _call(lib, aabbs, None, max_pairs)
        assert n == len(want)
        assert len(written) == max_pairs
        if max_pairs:
            got = {tuple(p) for p in written.tolist()}
            assert len(got) == max_pairs
            assert got <= {tuple(p) for p in want.tolist()}


def test_static_pairs_wide_group_ids(gpu_lib):
    # Group ids above 16 bits: ids that agree in their low 16 bits still keep
    # their boxes apart.
    lib = gpu_lib
    rng = np.random.default_rng(4)
    lo = rng.uniform(0, 3, (400, 3)).astype(np.float32)
    aabbs = np.concatenate([lo, lo + 0.8], axis=1)
    groups = rng.choice(np.array([5, 5 + 65536, 7, 7 + 3 * 65536, 0xfffffff0], np.uint32), 400)
    want = _brute_force(aabbs, groups)
    assert len(want) > 100
    for _ in range(2):
        np.testing.assert_array_equal(_static_pairs(lib, aabbs, groups, 8 * len(aabbs)), want)


def test_static_pairs_allocate_nothing(gpu_lib):
    # Neither the CUDA allocator nor torch's sees a byte change across calls
    # once the inputs and outputs exist.
    import torch
    lib = gpu_lib
    rng = np.random.default_rng(5)
    lo = rng.uniform(0, 20, (20000, 3)).astype(np.float32)
    aabbs = torch.from_numpy(np.concatenate([lo, lo + 0.5], axis=1)).cuda()
    pairs = torch.empty((200000, 2), dtype=torch.int32, device="cuda")
    count = torch.empty(1, dtype=torch.int32, device="cuda")
    args = (C.c_void_p(aabbs.data_ptr()), None, 20000, C.c_void_p(pairs.data_ptr()), 200000,
            C.c_void_p(count.data_ptr()), None)
    assert lib.npgpu_find_pairs_static(*args) == abi.OK      # set-up call
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    used0 = torch.cuda.memory_allocated()
    for _ in range(3):
        assert lib.npgpu_find_pairs_static(*args) == abi.OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_allocated() == used0
    n = int(count.cpu().numpy().view(np.uint32)[0])
    assert 0 < n <= 200000

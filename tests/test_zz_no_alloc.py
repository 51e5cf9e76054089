"""npgpu_find_pairs_static: the broad phase for callers that cannot allocate.

Callers that cannot call cudaMalloc (code running during CUDA graph capture,
real-time loops, hosts whose device memory belongs to another runtime's pool)
get the broad phase over device buffers they already own, with all scratch in
a fixed array inside the library. Its pairs must equal the world's own broad
phase (npgpu_get_pairs) on the same fat AABBs, call after call.
"""
import ctypes as C

import numpy as np
import pytest

from nphysics_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _static_pairs(lib, aabbs, groups, max_pairs):
    import torch
    d_aabb = torch.from_numpy(np.ascontiguousarray(aabbs, np.float32)).cuda()
    d_groups = torch.from_numpy(np.ascontiguousarray(groups, np.int32)).cuda() if groups is not None else None
    d_pairs = torch.full((max_pairs, 2), -1, dtype=torch.int32, device="cuda")
    d_count = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = lib.npgpu_find_pairs_static(C.c_void_p(d_aabb.data_ptr()),
                                     C.c_void_p(d_groups.data_ptr()) if d_groups is not None else None,
                                     len(aabbs), C.c_void_p(d_pairs.data_ptr()), max_pairs,
                                     C.c_void_p(d_count.data_ptr()), None)
    assert st == abi.OK, lib.npgpu_last_error(None)
    torch.cuda.synchronize()
    n = int(d_count.cpu().numpy().view(np.uint32)[0])
    assert n != 0xffffffff
    assert n <= max_pairs
    p = d_pairs[:n].cpu().numpy().view(np.uint32)
    order = np.lexsort((p[:, 1], p[:, 0]))
    return p[order]


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

"""The C++ mirror of the nphysics3d world API (nphysics_gb300/cpp) builds
against include/npgpu.h, and on a GPU steps the reference's pyramid scene to
the same poses, bit for bit, as the same scene loaded through the C ABI."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "pyramid_drop_in.cpp")


def compile_example(tmpdir):
    from nphysics_gb300 import build
    lib = build.build()
    exe = os.path.join(str(tmpdir), "pyramid_drop_in")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
                    lib, "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def test_cpp_mirror_compiles(tmp_path):
    assert os.path.exists(compile_example(tmp_path))


@pytest.mark.gpu
def test_cpp_mirror_steps_like_the_c_abi(gpu_lib, tmp_path):
    from nphysics_gb300 import scenes
    from nphysics_gb300.world import GpuWorld
    exe = compile_example(tmp_path)
    out = subprocess.run([exe, "30"], capture_output=True, text=True, check=True).stdout.split("\n")
    rows = [l.split() for l in out if l.strip()]
    assert len(rows) == 210
    got = np.array([[int(x, 16) for x in r[1:]] for r in rows], dtype=np.uint32).view(np.float32)
    sc = scenes.pyramid()
    w = GpuWorld.for_scene(sc)
    w.step(30)
    want = w.bodies()["position"][1:]
    np.testing.assert_array_equal(got, want)

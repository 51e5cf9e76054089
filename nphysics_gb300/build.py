"""Build recipe of libnpgpu.so (the CUDA rigid-body step behind include/npgpu.h).

Compiles each translation unit of csrc/ for sm_103a in parallel and links a
shared library into nphysics_gb300/_build/. Device code is compiled without
floating-point contraction (--fmad=false) and host code with
-ffp-contract=off, so that every operation rounds once, as in the oracle.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libnpgpu.so")
SOURCES = ["npgpu_world.cu", "k_bodies.cu", "k_cd.cu", "k_solve.cu", "k_static_pairs.cu", "k_mlp.cu"]
HEADERS = ["np_math.cuh", "world_dev.cuh", "dyn.cuh", "narrow.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return path


def _flags():
    return ARCH + ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-I" + os.path.join(HERE, "..", "include")]


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "npgpu.h")]
    return any(os.path.getmtime(d) > t for d in deps)


# The persistent solver kernel reads, after a grid barrier, data that other
# SMs wrote: its global loads bypass L1 (-dlcm=cg) so none is served stale.
EXTRA = {"k_solve.cu": ["-Xptxas", "-dlcm=cg"]}


def _compile(src):
    s = os.path.join(CSRC, src)
    o = os.path.join(OUT, src.replace(".cu", ".o"))
    if not _stale(o, s):
        return o, False
    cmd = [nvcc()] + _flags() + EXTRA.get(src, []) + ["-c", s, "-o", o + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    os.replace(o + ".tmp", o)
    return o, True


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    if force:
        for f in os.listdir(OUT):
            if f.endswith(".o"):
                os.remove(os.path.join(OUT, f))
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(_compile, SOURCES))
    objs = [o for o, _ in results]
    rebuilt = any(r for _, r in results) or not os.path.exists(LIB)
    if rebuilt:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)

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
# (source, object, extra flags): k_solve.cu is compiled twice, see EXTRA.
SOURCES = [("npgpu_world.cu", "npgpu_world.o", []), ("k_bodies.cu", "k_bodies.o", []), ("k_cd.cu", "k_cd.o", []),
           ("k_solve.cu", "k_solve.o", ["-DNPGPU_EXCHANGE_TU=0"]),
           ("k_solve.cu", "k_solve_exchange.o", ["-DNPGPU_EXCHANGE_TU=1", "-Xptxas", "-dlcm=cg"]),
           ("k_static_pairs.cu", "k_static_pairs.o", []), ("k_mlp.cu", "k_mlp.o", []),
           ("sortscan.cu", "sortscan.o", []), ("k_query.cu", "k_query.o", [])]
HEADERS = ["np_math.cuh", "world_dev.cuh", "dyn.cuh", "narrow.cuh", "mlp.cuh", "sortscan.cuh"]
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


# The kernels whose blocks exchange data through global memory within one
# launch (the persistent solvers, the dataflow colouring, the islands'
# union-find, the cluster solvers) read, after a barrier or a flag, data that
# other SMs wrote: their translation unit (k_solve.cu with
# NPGPU_EXCHANGE_TU=1) has its global loads bypass L1 (-dlcm=cg) so none is
# served stale. The other kernels keep L1 caching.


def _compile(entry):
    src, obj, extra = entry
    s = os.path.join(CSRC, src)
    o = os.path.join(OUT, obj)
    if not _stale(o, s):
        return o, False
    cmd = [nvcc()] + _flags() + extra + ["-c", s, "-o", o + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src} ({obj}):\n{r.stdout}\n{r.stderr}")
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

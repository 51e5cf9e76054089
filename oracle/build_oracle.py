"""Build recipe of the CPU oracle (test infrastructure only).

Compiles oracle/oracle_capi.cpp into oracle/_build/liboracle.so with strict
IEEE arithmetic (-ffp-contract=off: no fused multiply-add on any host
architecture, so x86_64 and aarch64 produce the same bits).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "oracle_capi.cpp")]
HEADERS = [os.path.join(HERE, f) for f in ("ref_math.hpp", "ref_ccd.hpp", "ref_world.hpp")] + [
    os.path.join(HERE, "..", "include", "npgpu.h")
]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in SOURCES + HEADERS)


def build(force=False):
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-Wall", "-Wno-unused-function", "-o", LIB + ".tmp"] + SOURCES
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))

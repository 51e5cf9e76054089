"""The C ABI library loads and exports every entry point include/npgpu.h
declares, and the ctypes mirror has the header's struct layouts (no GPU)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from nphysics_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "npgpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(npgpu_[a-z_0-9]+)\s*\(", src)))


@pytest.fixture(scope="module")
def built():
    from nphysics_gb300 import build
    return build.build()


def test_library_exports_every_declared_entry_point(built):
    names = declared_functions()
    assert set(names) == set(abi.EXPORTED)
    lib = C.CDLL(built)
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", built], capture_output=True, text=True, check=True).stdout
    for n in names:
        assert re.search(rf"\bT {n}\b", out), n


def test_version_and_default_params_without_gpu(built):
    lib = abi.load_library(built)
    assert lib.npgpu_abi_version() == abi.NPGPU_ABI_VERSION
    p = abi.Params()
    lib.npgpu_default_params(C.byref(p))
    ref = abi.default_params()
    for name, _ in abi.Params._fields_:
        assert getattr(p, name) == pytest.approx(getattr(ref, name)), name


def test_create_without_a_device_reports_an_error(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = abi.load_library(built)
    st = C.c_int(-1)
    w = lib.npgpu_create(C.byref(abi.default_params()), (C.c_float * 3)(0, -9.81, 0), 8, 8, 64, C.byref(st))
    assert not w
    assert st.value == abi.ERR_CUDA
    assert b"device" in lib.npgpu_last_error(None)


def test_struct_layouts_match_the_header():
    prog = r"""
#include <stdio.h>
#include <stddef.h>
#include "npgpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(npgpu_handle), sizeof(npgpu_body_desc),
         sizeof(npgpu_collider_desc), sizeof(npgpu_params), sizeof(npgpu_counters), sizeof(npgpu_contact),
         offsetof(npgpu_counters, residual));
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "sz.c")
        exe = os.path.join(d, "sz")
        open(src, "w").write(prog)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        got = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    want = [C.sizeof(abi.Handle), C.sizeof(abi.BodyDesc), C.sizeof(abi.ColliderDesc), C.sizeof(abi.Params),
            C.sizeof(abi.Counters), C.sizeof(abi.Contact), abi.Counters.residual.offset]
    assert got == want


def test_missing_library_fails_loudly(tmp_path):
    # No CPU fallback: the product without its built library raises.
    with pytest.raises(RuntimeError, match="not built"):
        abi.load_library(str(tmp_path / "libnpgpu.so"))


def test_product_never_uses_the_oracle():
    # The CPU oracle is test infrastructure: no module, kernel or header of
    # the product imports, includes or loads it.
    pkg = os.path.join(ROOT, "nphysics_gb300")
    bad = []
    for dirpath, _, files in os.walk(pkg):
        if "_build" in dirpath or "__pycache__" in dirpath:
            continue
        for f in files:
            if not f.endswith((".py", ".cu", ".cuh", ".hpp", ".cpp", ".h")):
                continue
            path = os.path.join(dirpath, f)
            for n, line in enumerate(open(path, encoding="utf-8"), 1):
                code = line.split("#")[0] if f.endswith(".py") else line.split("//")[0]
                if re.search(r"\b(from|import)\s+oracle\b|#include\s*[<\"][^>\"]*oracle|liboracle|oracle_py|ref_world",
                             code):
                    bad.append(f"{os.path.relpath(path, ROOT)}:{n}: {line.strip()}")
    assert not bad, bad
    hdr = open(HEADER).read()
    assert "oracle" not in hdr


def test_rust_binding_declares_every_entry_point():
    # The reference-side binding (the Rust crate's extern "C" block) names
    # every function include/npgpu.h declares.
    text = open(os.path.join(ROOT, "rust", "nphysics3d-gpu", "src", "ffi.rs")).read()
    i = text.index('extern "C" {')
    block = text[i:text.index("\n}", i)]
    missing = [f for f in declared_functions() if re.search(r"\bfn " + f + r"\(", block) is None]
    assert not missing, missing


def test_every_entry_point_cites_the_reference():
    # Each group of declarations (a paragraph of the header) has a comment that
    # names the reference interface it replaces (a src/...rs file:line) or says
    # that the reference has no counterpart.
    src = open(HEADER).read()
    uncited, seen = [], set()
    for para in re.split(r"\n\s*\n", src):
        names = re.findall(r"\b(npgpu_[a-z_0-9]+)\s*\(", re.sub(r"/\*.*?\*/", "", para, flags=re.S))
        if not names:
            continue
        seen.update(names)
        comments = " ".join(re.findall(r"/\*.*?\*/", para, flags=re.S))
        if not (".rs" in comments or "counterpart" in comments.lower()):
            uncited += names
    assert not uncited, uncited
    assert set(declared_functions()) <= seen

"""The C-ABI library builds, loads without a GPU and exports every entry point
declared in include/fgpu.h (no compute calls here)."""
import os
import re
import subprocess

import pytest

from tests.conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "fgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fgpu_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "fgpu_assemble_matrix" in names and "fgpu_solve_cg" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(fgpu_lib):
    from feelpp_gb300 import _ffi
    out = subprocess.run(["nm", "-D", "--defined-only", _ffi.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s+(fgpu_\w+)", out))
    missing = [n for n in declared_symbols() if n not in exported]
    assert not missing, missing
    for n in declared_symbols():
        assert hasattr(fgpu_lib, n)


def test_ffi_signatures_cover_header():
    from feelpp_gb300 import _ffi
    assert set(declared_symbols()) == set(_ffi.SIGNATURES)


def test_create_without_gpu_fails_cleanly(fgpu_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import ctypes as C
    from feelpp_gb300 import _ffi
    h = C.c_void_p()
    cfg = _ffi.Config(0, None, 0, 1)
    rc = fgpu_lib.fgpu_create(C.byref(cfg), C.byref(h))
    assert rc == 2 and not h.value  # FGPU_ERR_CUDA, no context


def test_oracle_is_not_linked_by_the_product():
    from feelpp_gb300 import _ffi
    out = subprocess.run(["ldd", _ffi.LIB_PATH], capture_output=True, text=True).stdout
    assert "oracle" not in out
    for dirpath, _, files in os.walk(os.path.join(ROOT, "feelpp_gb300")):
        for f in files:
            if f.endswith((".py", ".cu", ".cpp", ".h")):
                txt = open(os.path.join(dirpath, f)).read()
                assert "pyoracle" not in txt and "liboracle" not in txt and "import oracle" not in txt, f

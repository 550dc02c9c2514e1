"""The C-ABI library builds, loads and exports every entry point that
include/flipgpu.h declares (no device calls: this runs without a GPU)."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "flipgpu.h")).read()
    return sorted(set(re.findall(r"\b(flip(?:gpu|unet|batch)_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_entry_points():
    names = declared_symbols()
    for must in ("flipgpu_create", "flipgpu_sort", "flipgpu_p2g", "flipgpu_g2p",
                 "flipgpu_solve", "flipgpu_correct", "flipgpu_step", "flipgpu_mesh",
                 "flipgpu_implicit", "flipunet_train_step", "flipgpu_set_warm_start"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from flip3d_gb300 import build
    path = build.build()
    lib = C.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_bindings_cover_the_header():
    from flip3d_gb300 import gpu
    assert set(declared_symbols()) == set(gpu.SIGNATURES)

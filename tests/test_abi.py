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


def test_python_structures_match_the_header(tmp_path):
    """Every ctypes structure of the binding has the C layout of its
    header struct: field offsets and total size, from a program compiled
    against include/flipgpu.h."""
    import shutil
    import subprocess

    from flip3d_gb300 import gpu
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    structs = {"FlipGpuParams": gpu.Params, "FlipGpuSolveStats": gpu.SolveStats,
               "FlipSceneObject": gpu.SceneObject, "FlipCheckpoint": gpu.Checkpoint}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "flipgpu.h"',
             "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    c_layout = {}
    for line in out.splitlines():
        cname, what, value = line.split()
        c_layout[(cname, what)] = int(value)
    for cname, py in structs.items():
        assert C.sizeof(py) == c_layout[(cname, "size")], cname
        for field, _ in py._fields_:
            assert getattr(py, field).offset == c_layout[(cname, field)], (cname, field)

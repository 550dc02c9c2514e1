"""An unmodified copy of the reference driver (src/flip3D.cpp, src/main.cpp)
compiles and links against the GPU shim in place of the reference's
sorter/mapper/solver/corrector/mesher/implicit sources (and the marching
cubes they use). Needs the reference tree; skipped
where it is absent. Builds only (running needs a GPU)."""
import os
import subprocess

import pytest

REF = "/root/reference/src"
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference tree not present")
def test_reference_driver_links_against_shim(tmp_path):
    from flip3d_gb300 import build
    build.build_shim()
    here = os.path.join(ROOT, "flip3d_gb300")
    shim = os.path.join(here, "shim")
    force = []
    for h in ("sorter.h", "mapper.h", "solver.h", "corrector.h", "mesher.h", "implicit.h"):
        force += ["-include", os.path.join(shim, h)]
    common = ["-O1", "-w", "-fopenmp", "-I", REF, "-I", os.path.join(REF, "rchandra"),
              "-include", "cmath", "-include", "limits", "-include", "vector", "-include", "map"]
    objs = []
    # the driver itself, with the shim's declarations in force
    for src in ("flip3D.cpp", "main.cpp"):
        o = str(tmp_path / (src + ".o"))
        subprocess.check_call(["g++", *common, *force, "-c", os.path.join(REF, src), "-o", o])
        objs.append(o)
    # the reference's files that stay on the host (not the replaced hot path)
    for src in ("utility.cpp", "kernel.cpp", "exporter.cpp", "write_bmp.cpp"):
        o = str(tmp_path / (os.path.basename(src) + ".o"))
        subprocess.check_call(["g++", *common, "-include", "algorithm", *force, "-c",
                               os.path.join(REF, src), "-o", o])
        objs.append(o)
    exe = str(tmp_path / "flip3d_gpu")
    subprocess.check_call(["g++", "-fopenmp", "-o", exe, *objs, "-L", here, "-lflip3d_shim",
                           "-lflipgpu", f"-Wl,-rpath,{here}"])
    assert os.path.exists(exe)

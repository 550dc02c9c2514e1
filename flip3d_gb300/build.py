"""Build libflipgpu.so (the CUDA kernels and the C ABI) in-tree for sm_103a.

Each translation unit compiles in parallel with nvcc; the objects link into
flip3d_gb300/libflipgpu.so. Simulation kernels build with -fmad=false: the
reference's float expressions round after every multiply and add, and fusing
them would change results.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libflipgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = ["api.cu", "k_sort.cu", "k_particles.cu", "k_grid.cu", "k_pcg.cu", "k_mesh.cu", "k_unet.cu",
           "k_conv_tc.cu", "k_scene.cu", "checkpoint.cu", "export.cu", "k_preview.cu",
           "autotune.cu",
           "noalloc_sort.cu"]
FLAGS = {name: ["-fmad=false"] for name in SOURCES}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
           *FLAGS.get(src, []), "-I", os.path.join(HERE, "..", "include"),
           "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(-4, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stderr}")
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)
    return obj


def stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "flipgpu.h"))
    deps.append(os.path.join(HERE, "..", "include", "flip_rng.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


SHIM_LIB = os.path.join(HERE, "libflip3d_shim.so")


def build_shim(force: bool = False) -> str:
    """libflip3d_shim.so: the reference's sorter/mapper/solver/corrector call
    surface on top of libflipgpu.so (host C++, g++)."""
    lib = build(force=force)
    src = os.path.join(HERE, "shim", "shim.cpp")
    deps = [src] + [os.path.join(HERE, "shim", f) for f in os.listdir(os.path.join(HERE, "shim"))
                    if f.endswith(".h")]
    if (not force and os.path.exists(SHIM_LIB)
            and all(os.path.getmtime(d) <= os.path.getmtime(SHIM_LIB) for d in deps + [lib])):
        return SHIM_LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", SHIM_LIB + ".tmp", src,
           "-I", os.path.join(HERE, "shim", "compat"), "-L", HERE, "-lflipgpu",
           "-Wl,-rpath,$ORIGIN"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"shim build failed:\n{res.stderr}")
    os.replace(SHIM_LIB + ".tmp", SHIM_LIB)
    return SHIM_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_shim(force="--force" in sys.argv))

"""The C++ shim (the reference's sorter/mapper/solver/corrector signatures
over libflipgpu) driven by a native program the way src/flip3D.cpp calls it,
compared with the CPU oracle on the same inputs."""
import os
import subprocess

import numpy as np
import pytest

from flip3d_gb300 import scenes

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_driver(tmp):
    from flip3d_gb300 import build
    build.build_shim()
    exe = os.path.join(tmp, "shim_driver")
    here = os.path.join(ROOT, "flip3d_gb300")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-o", exe,
                           os.path.join(ROOT, "tests", "native", "shim_driver.cpp"),
                           "-I", os.path.join(here, "shim"), "-I", os.path.join(here, "shim", "compat"),
                           "-L", here, "-lflip3d_shim", "-lflipgpu", f"-Wl,-rpath,{here}"])
    return exe


def test_shim_drives_the_gpu_like_the_reference(tmp_path):
    from oracle import pyoracle as orc
    g = np.load(os.path.join(ROOT, "tests", "golden", "components_n16.npz"))
    n = int(g["n"])
    pos, vel, nrm, typ, dens = g["pos"], g["vel"], g["nrm"], g["type"], g["dens"]
    np_ = pos.shape[0]
    rng = np.random.default_rng(3)
    grid = [rng.normal(0, 1, (n + 1) * n * n).astype(np.float32) for _ in range(3)]
    sg = np.load(os.path.join(ROOT, "tests", "golden", "solver_n16.npz"))
    b, x0 = sg["b"], sg["x0"]
    q = rng.uniform(0.05, 0.95, (5, 3)).astype(np.float32)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([n, np_], np.int32).tofile(f)
        for a in (pos, vel, nrm):
            a.astype(np.float32).tofile(f)
        typ.astype(np.uint8).tofile(f)
        dens.astype(np.float32).tofile(f)
        for a in grid:
            a.tofile(f)
        b.astype(np.float32).tofile(f)
        x0.astype(np.float32).tofile(f)
        np.array([q.shape[0]], np.int32).tofile(f)
        q.tofile(f)
    out = tmp_path / "out.bin"
    subprocess.check_call([build_driver(str(tmp_path)), str(inp), str(out)])
    raw = open(out, "rb").read()
    off = 0

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a

    nc, nf = n ** 3, (n + 1) * n * n
    cs, perm = take(np.uint32, nc + 1), take(np.uint32, np_)
    assert np.array_equal(cs, g["cell_start"]) and np.array_equal(perm, g["perm"])
    nbn = int(take(np.int32, 1)[0])
    nb = take(np.uint32, nbn)
    i, j, k = n // 2, n // 3, n // 2
    want = [perm[a] for si in range(i - 1, i + 2) for sj in range(j - 1, j + 2)
            for sk in range(k - 1, k + 2)
            for a in range(cs[(si * n + sj) * n + sk], cs[(si * n + sj) * n + sk + 1])]
    assert list(nb) == want
    A, L = take(np.uint8, nc), take(np.float32, nc)
    assert np.array_equal(A, g["A"]) and np.array_equal(L, g["L"])
    u = [take(np.float32, nf) for _ in range(3)]
    for c in range(3):
        assert np.array_equal(u[c], g[f"u{c}"])
    fetched = take(np.float32, 15).reshape(5, 3)
    assert np.array_equal(fetched, orc.g2p(n, q, np.ones(5, np.uint8), grid))
    g2p = take(np.float32, 3 * np_).reshape(np_, 3)
    ref = orc.g2p(n, pos, typ, grid)
    ub = (np.float32(n) * pos[:, 2]) > np.float32(n - 0.5)
    assert np.array_equal(g2p[~ub], ref[~ub])
    x, bo = take(np.float32, nc), take(np.float32, nc)
    prm = orc.params(n, orc.PRECOND_REF)
    xr, br, _, _, _ = orc.solve(prm, A, L, x0, b)
    assert np.array_equal(bo, br)
    assert np.abs(x - xr).max() <= 1e-5 * np.abs(xr).max()
    cpos = take(np.float32, 3 * np_).reshape(np_, 3)
    cvel = take(np.float32, 3 * np_).reshape(np_, 3)
    fl = typ == 1
    assert np.array_equal(cpos, g["corr_pos"])
    assert np.array_equal(cvel[fl], g["corr_vel"][fl])
    # resample at q[0]: the lists of the positions before the move over the
    # particles' current (corrected) data, as the reference's sorter does
    ru = take(np.float32, 3)
    rr = orc.resample(n, g["corr_pos"], g["corr_vel"], typ, cs, perm, q[0],
                      np.zeros(3, np.float32), 1.0 / n)
    assert np.array_equal(ru, rr)
    phi = take(np.float64, 1)
    assert np.array_equal(phi, orc.implicit(n, g["corr_pos"], typ, cs, perm, q[:1]))
    nv, nfc = (int(v) for v in take(np.int64, 2))
    mv, mn = take(np.float64, 3 * nv), take(np.float64, 3 * nv)
    mf = take(np.int32, 3 * nfc)
    om = orc.mesh(n, g["corr_pos"], typ, cs, perm)
    assert np.array_equal(mv, om["vertices"]) and np.array_equal(mn, om["normals"])
    assert np.array_equal(mf, om["faces"])
    assert off == len(raw)

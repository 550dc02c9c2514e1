"""The reference's checkpoint layout (saveState/loadState,
src/flip3D.cpp:453-578) against a file the reference itself wrote
(tests/golden/checkpoint_n32.npz: its init + saveState at N=32, made by
tests/golden/make_golden.py). The reader and writer are host code of
libflipgpu.so and run without a GPU."""
import hashlib
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(HERE, "golden", "checkpoint_n32.npz"))


@pytest.fixture(scope="module")
def gpu():
    from flip3d_gb300 import gpu as g
    g.load()
    return g


def _state(g):
    return {"pos": g["pos"], "vel": g["vel"], "nrm": g["nrm"], "type": g["type"],
            "dens": g["dens"], "press": g["press"], "wall_normal": g["wall_normal"],
            "max_dens": float(g["max_dens"]), "pour_time": int(g["pour_time"]),
            "pour_pos": tuple(float(v) for v in g["pour_pos"]), "pour_rad": float(g["pour_rad"])}


def test_writer_reproduces_the_reference_file(gpu, golden, tmp_path):
    """Written from the reference file's content (visible left to the
    writer's default), the bytes equal the reference's, apart from the
    fields the reference leaves undefined (tmp, remove, the normals of
    cells no particle visits), which both sides hold at zero."""
    path = str(tmp_path / "ours.dat")
    n = int(golden["n"])
    gpu.checkpoint_write(path, n, _state(golden))
    raw = open(path, "rb").read()
    assert len(raw) == int(golden["file_bytes"])
    assert hashlib.sha256(raw).hexdigest() == str(golden["canonical_sha256"])


def test_reader_recovers_the_content(gpu, golden, tmp_path):
    path = str(tmp_path / "ours.dat")
    n = int(golden["n"])
    gpu.checkpoint_write(path, n, _state(golden))
    got = gpu.checkpoint_read(path, n)
    assert got["count"] == int(golden["count"])
    for k in ("pos", "vel", "nrm", "type", "visible", "dens", "press", "wall_normal"):
        assert np.array_equal(got[k], golden[k]), k
    assert got["max_dens"] == float(golden["max_dens"])
    assert got["pour_time"] == int(golden["pour_time"])
    assert got["pour_rad"] == np.float32(golden["pour_rad"])


def test_reader_rejects_a_wrong_grid_size(gpu, golden, tmp_path):
    path = str(tmp_path / "ours.dat")
    gpu.checkpoint_write(path, int(golden["n"]), _state(golden))
    with pytest.raises(gpu.FlipGpuError):
        gpu.checkpoint_read(path, 16)


def test_reader_checks_the_capacity_of_every_particle_array(gpu, golden, tmp_path):
    """c->count is the capacity of each per-particle array given: a file with
    more particles is rejected whichever of them is set (ETOOBIG, nothing
    written), and a negative count is an invalid argument."""
    import ctypes as C
    path = str(tmp_path / "ours.dat")
    n = int(golden["n"])
    gpu.checkpoint_write(path, n, _state(golden))
    lib = gpu.load()
    small = int(golden["count"]) - 1
    for key, dt, width in (("type", np.uint8, 1), ("dens", np.float32, 1),
                           ("nrm", np.float32, 3), ("visible", np.uint8, 1)):
        buf = np.full(small * width, 7, dt)
        c = gpu.Checkpoint()
        c.n, c.count = n, small
        setattr(c, key, buf.ctypes.data)
        assert lib.flipgpu_checkpoint_read(path.encode(), C.byref(c)) == -7, key
        assert (buf == 7).all(), key
    c = gpu.Checkpoint()
    c.n, c.count = n, -1
    assert lib.flipgpu_checkpoint_read(path.encode(), C.byref(c)) == -1
    # grid sections only: no per-particle array, any capacity
    press = np.zeros(n ** 3, np.float32)
    c = gpu.Checkpoint()
    c.n, c.count = n, 0
    c.press = press.ctypes.data
    assert lib.flipgpu_checkpoint_read(path.encode(), C.byref(c)) == 0
    assert c.count == int(golden["count"])
    assert np.array_equal(press, golden["press"])

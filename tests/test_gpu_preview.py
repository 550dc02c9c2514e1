"""flipgpu_preview + flipgpu_write_bmp against the BMPs the reference's own
write_frame wrote for the same particles (tests/golden/preview_n32.npz,
made by tests/golden/make_golden.py): byte-identical files."""
import hashlib
import os
import time

import numpy as np
import pytest

from flip3d_gb300 import scenes

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gpu():
    from flip3d_gb300 import gpu as g
    g.load()
    return g


@pytest.mark.parametrize("tag,make", [("pool_sphere", lambda n: scenes.pool_sphere(n, seed=0)),
                                      ("random_s5", lambda n: scenes.random_scene(n, 5))])
def test_preview_bmp_is_the_references(gpu, tmp_path, tag, make):
    g = np.load(os.path.join(HERE, "golden", "preview_n32.npz"))
    sc = make(int(g["n"]))
    sim = gpu.Simulation(gpu.default_params(sc.n, sc.count + 8))
    sim.set_scene(sc)
    path = str(tmp_path / "frame.bmp")
    img = sim.write_preview(path)
    raw = open(path, "rb").read()
    assert len(raw) == int(g[f"{tag}_bytes"])
    assert int((np.frombuffer(raw[54:], np.uint8) > 0).sum()) == int(g[f"{tag}_covered"])
    assert hashlib.sha256(raw).hexdigest() == str(g[f"{tag}_sha256"])
    assert (img[..., 3] == 255).all()


def test_preview_at_scale(gpu):
    """N=256 sphere into pool (34.8M particles) seeded on the device: the
    preview runs in milliseconds; the result is deterministic."""
    sc_objs = scenes.sphere_into_pool(32).objects  # object list only; seeded at N=256 below
    n = 256
    wall = 1.0 / n
    objs = [scenes.Box((wall, wall, wall), (1 - wall, 0.25, 1 - wall)),
            scenes.Sphere((0.5, 0.75, 0.5), 0.15, (0.0, -2.0, 0.0))]
    assert len(sc_objs) == len(objs)
    sim = gpu.Simulation(gpu.default_params(n, 36_000_000))
    sim.seed_scene(objs, 0)
    a = sim.preview()
    t0 = time.perf_counter()
    b = sim.preview()
    ms = 1e3 * (time.perf_counter() - t0)
    print(f"N=256 preview of {sim.np} particles: {ms:.2f} ms (with the 2.9 MB download)")
    assert np.array_equal(a, b)

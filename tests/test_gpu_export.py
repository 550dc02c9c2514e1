"""flipgpu_export_mesh: the device mesh downloaded asynchronously and
written on a host thread gives the same files as the host writers on the
mesh flipgpu_get_mesh returns (those are pinned to the reference's own
exporter by tests/test_export.py)."""
import time

import numpy as np
import pytest

from flip3d_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from flip3d_gb300 import gpu as g
    g.load()
    return g


@pytest.mark.parametrize("n", [32, 64])
def test_async_export_equals_host_writers(gpu, tmp_path, n):
    sc = scenes.pool_sphere(n, seed=2)
    sim = gpu.Simulation(gpu.default_params(n, sc.count + 64, rel_tol=1e-6,
                                            solve_mode=gpu.SOLVE_FAST,
                                            precond=gpu.PRECOND_JACOBI, seed=2))
    sim.seed_scene(sc.objects, 2)
    sim.calibrate_max_density()
    sim.step()
    m = sim.mesh()
    wt = np.float32(1.0 / n)
    t0 = time.perf_counter()
    sim.export_mesh(str(tmp_path / "dev"), 3, float(wt), wait=False)
    t_enqueue = time.perf_counter() - t0
    sim.export_wait()
    t_all = time.perf_counter() - t0
    host_obj, host_sc = str(tmp_path / "h.obj"), str(tmp_path / "h.sc")
    gpu.write_mesh_files(host_obj, host_sc, m["vertices"], m["normals"], m["faces"], float(wt))
    print(f"n={n}: {m['vertices'].shape[0]} vertices, export enqueued in "
          f"{1e3 * t_enqueue:.2f} ms, written after {1e3 * t_all:.1f} ms")
    assert open(tmp_path / "dev" / "obj" / "3_scene.obj", "rb").read() == open(host_obj, "rb").read()
    assert open(tmp_path / "dev" / "sunflow" / "3_scene.sc", "rb").read() == \
        open(host_sc, "rb").read()
    assert not (tmp_path / "dev" / "sunflow" / "template.sc").exists()
    sim.export_mesh(str(tmp_path / "dev2"), 4, float(wt), formats=gpu.EXPORT_SUNFLOW,
                    sunflow_template="% scene settings\n")
    assert open(tmp_path / "dev2" / "sunflow" / "template.sc").read() == "% scene settings\n"
    assert not (tmp_path / "dev2" / "obj").exists()


def test_export_without_mesh_fails_cleanly(gpu, tmp_path):
    sc = scenes.pool_sphere(16, seed=0)
    sim = gpu.Simulation(gpu.default_params(16, sc.count + 8))
    sim.seed_scene(sc.objects, 0)
    with pytest.raises(gpu.FlipGpuError):
        sim.export_mesh(str(tmp_path / "x"), 0, 1 / 16)

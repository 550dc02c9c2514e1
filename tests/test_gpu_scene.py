"""Scene setup on the device (flipgpu_seed_scene) against the host
generator (flip3d_gb300/scenes.py:build, the restatement of flip3D::init's
seeding with the counter-based jitter): the same particles bit for bit, in
the same order, and the same first steps (which also compares the wall
normals and the wall lists the advection walks)."""
import numpy as np
import pytest

from flip3d_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from flip3d_gb300 import gpu as g
    g.load()
    return g


def _sim(gpu, n, cap, seed):
    s = gpu.Simulation(gpu.default_params(n, cap, rel_tol=1e-6, solve_mode=gpu.SOLVE_FAST,
                                          precond=gpu.PRECOND_JACOBI, seed=seed))
    return s


@pytest.mark.parametrize("make,n,seed", [
    (scenes.pool_sphere, 32, 0), (scenes.dam_break, 48, 3), (scenes.sphere_into_pool, 32, 1),
    (scenes.random_scene, 32, 7), (scenes.random_scene, 24, 11)])
def test_device_seeding_matches_host_scene(gpu, make, n, seed):
    sc = make(n, seed)
    host = _sim(gpu, n, sc.count + 16, seed)
    host.set_scene(sc)
    dev = _sim(gpu, n, sc.count + 16, seed)
    dev.seed_scene(sc.objects, seed)
    assert dev.np == sc.count
    hp = host.get_particles()
    dp = dev.get_particles()
    for a, b in zip(hp, dp):
        assert np.array_equal(a, b)
    for s in (host, dev):
        s.calibrate_max_density()
    for _ in range(2):
        a, b = host.step(), dev.step()
        assert a.iterations == b.iterations
    for x, y in zip(host.get_particles(), dev.get_particles()):
        assert np.array_equal(x, y)


def test_device_seeding_rejects_a_full_handle(gpu):
    sc = scenes.pool_sphere(16, 0)
    s = _sim(gpu, 16, sc.count // 2, 0)
    with pytest.raises(gpu.FlipGpuError):
        s.seed_scene(sc.objects, 0)

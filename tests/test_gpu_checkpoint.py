"""flipgpu_save_state / flipgpu_load_state: the wall-normal grid computed
on the device equals the one the reference's compute_wall_normal wrote into
its own checkpoint (tests/golden/checkpoint_n32.npz; the cube walls make it
independent of the liquid), and a state saved after some steps and loaded
into a fresh handle continues with identical steps."""
import os

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


def _sim(gpu, sc, seed=5):
    s = gpu.Simulation(gpu.default_params(sc.n, sc.count + 64, rel_tol=1e-6,
                                          solve_mode=gpu.SOLVE_FAST,
                                          precond=gpu.PRECOND_JACOBI, seed=seed))
    return s


def test_saved_wall_normals_match_the_reference(gpu, tmp_path):
    g = np.load(os.path.join(HERE, "golden", "checkpoint_n32.npz"))
    sc = scenes.pool_sphere(32, seed=1)
    sim = _sim(gpu, sc)
    sim.seed_scene(sc.objects, 1)
    sim.calibrate_max_density()
    path = str(tmp_path / "s.dat")
    sim.save_state(path)
    got = gpu.checkpoint_read(path, 32)
    assert np.array_equal(got["wall_normal"], g["wall_normal"])
    pos, vel, dens, typ = sim.get_particles()
    assert np.array_equal(got["pos"], pos) and np.array_equal(got["type"], typ)
    assert np.array_equal(got["visible"], (typ == 1).astype(np.uint8))


@pytest.mark.parametrize("arith", [0, 1])
def test_save_load_continues_identically(gpu, tmp_path, arith):
    sc = scenes.dam_break(32, seed=2)
    a = gpu.Simulation(gpu.default_params(sc.n, sc.count + 64, rel_tol=1e-6,
                                          solve_mode=gpu.SOLVE_FAST, precond=gpu.PRECOND_JACOBI,
                                          seed=9, arith=arith))
    a.set_scene(sc)
    a.calibrate_max_density()
    for _ in range(3):
        a.step()
    path = str(tmp_path / "a.dat")
    a.save_state(path, pour_time=200, pour_pos=(0.2, 0.3), pour_rad=0.1)
    b = gpu.Simulation(gpu.default_params(sc.n, sc.count + 64, rel_tol=1e-6,
                                          solve_mode=gpu.SOLVE_FAST, precond=gpu.PRECOND_JACOBI,
                                          seed=9, arith=arith))
    pour = b.load_state(path)
    assert pour["pour_time"] == 200 and pour["pour_rad"] == np.float32(0.1)
    b.set_step(3)
    for x, y in zip(a.get_particles(), b.get_particles()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.get_grid()[3], b.get_grid()[3])  # pressure
    for _ in range(2):
        sa, sb = a.step(), b.step()
        assert sa.iterations == sb.iterations
    for x, y in zip(a.get_particles(), b.get_particles()):
        assert np.array_equal(x, y)

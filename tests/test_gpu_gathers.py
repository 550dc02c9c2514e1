"""The FAST-arithmetic gathers the step runs (density and P2G with one
thread per cell, the corrector's spring and resample without per-thread
near lists) against the per-particle kernels (FLIPGPU_GATHER=particle): the
same sums in the same order with the same arithmetic, so whole steps are
bit-identical, on an ordinary scene and on one with crowded cells (more
particles than a thread's register group)."""
import os

import numpy as np
import pytest

from flip3d_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from flip3d_gb300 import gpu as g
    g.load()
    return g


def crowded_scene(n, seed):
    sc = scenes.dam_break(n, seed=seed)
    rng = np.random.default_rng(seed)
    fl = np.flatnonzero(sc.type == 1)
    pick = rng.choice(fl, size=min(4000, fl.size // 4), replace=False)
    lo = np.array([0.15, 0.1, 0.4], np.float32)
    sc.pos[pick] = lo + rng.uniform(0, 1, (pick.size, 3)).astype(np.float32) * \
        np.array([2.0 / n, 2.0 / n, 3.0 / n], np.float32)
    return sc


def run(gpu, sc, mode, steps=3):
    if mode:
        os.environ["FLIPGPU_GATHER"] = mode
    try:
        sim = gpu.Simulation(gpu.default_params(sc.n, sc.count, rel_tol=1e-6, seed=5,
                                                solve_mode=gpu.SOLVE_FAST,
                                                precond=gpu.PRECOND_MG, arith=gpu.ARITH_FAST))
        sim.set_scene(sc)
        sim.calibrate_max_density()
        for _ in range(steps):
            assert sim.step().status == 0
        pos, vel, dens, _ = sim.get_particles()
        u, A, L, p, _ = sim.get_grid()
        sim.close()
        return [pos, vel, dens, *u, A, L, p]
    finally:
        os.environ.pop("FLIPGPU_GATHER", None)


@pytest.mark.parametrize("crowd", [False, True])
def test_fast_gathers_equal_the_per_particle_kernels(gpu, crowd):
    n = 48
    sc = crowded_scene(n, 3) if crowd else scenes.pool_sphere(n, seed=3)
    a = run(gpu, sc, "particle")
    b = run(gpu, sc, None)
    names = ["pos", "vel", "dens", "u0", "u1", "u2", "A", "L", "press"]
    bad = [nm for nm, x, y in zip(names, a, b) if not np.array_equal(x, y)]
    assert not bad, bad

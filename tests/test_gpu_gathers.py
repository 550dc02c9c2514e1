"""The FAST-arithmetic gathers the step runs (P2G with one thread per face
cell, the corrector's spring and resample without per-thread near lists)
against the per-particle kernels (FLIPGPU_GATHER=particle), stage by stage
from the same state: the same sums in the same order, so bit-identical, on
an ordinary scene and on one with crowded cells."""
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
    sc.vel[pick] = rng.normal(0, 0.5, (pick.size, 3)).astype(np.float32)
    return sc


def params(gpu, sc):
    return gpu.default_params(sc.n, sc.count, rel_tol=1e-6, seed=5, solve_mode=gpu.SOLVE_FAST,
                              precond=gpu.PRECOND_MG, arith=gpu.ARITH_FAST)


def stages(gpu, sc, state, mode):
    """density, P2G and the corrector, each from `state` (positions,
    velocities) with the gathers of `mode`."""
    if mode:
        os.environ["FLIPGPU_GATHER"] = mode
    try:
        pos, vel = state
        out = {}
        sim = gpu.Simulation(params(gpu, sc))
        sim.set_particles(pos, sc.type, vel, sc.nrm)
        sim.calibrate_max_density()
        sim.set_particles(pos, sc.type, vel, sc.nrm)
        sim.sort()
        sim.compute_density()
        out["dens"] = sim.get_particles()[2]
        sim.p2g()
        u = sim.get_grid()[0]
        out.update(u0=u[0], u1=u[1], u2=u[2])
        sim.set_step(3)
        sim.correct()
        p, v, _, _ = sim.get_particles()
        out.update(pos=p, vel=v)
        sim.close()
        return out
    finally:
        os.environ.pop("FLIPGPU_GATHER", None)


@pytest.mark.parametrize("crowd", [False, True])
def test_fast_gathers_against_the_per_particle_kernels(gpu, crowd):
    n = 48
    sc = crowded_scene(n, 3) if crowd else scenes.pool_sphere(n, seed=3)
    # a state with moving particles: two steps of the benchmark's configuration
    sim = gpu.Simulation(params(gpu, sc))
    sim.set_scene(sc)
    sim.calibrate_max_density()
    for _ in range(2):
        assert sim.step().status == 0
    pos, vel, _, _ = sim.get_particles()
    sim.close()
    a = stages(gpu, sc, (pos, vel), "particle")
    b = stages(gpu, sc, (pos, vel), None)
    b2 = stages(gpu, sc, (pos, vel), None)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(b[k], b2[k]), k      # deterministic


@pytest.mark.parametrize("crowd", [False, True])
def test_fast_cell_lists_put_the_lower_half_first(gpu, crowd):
    """FAST arithmetic lists each cell's particles below its mid-plane in z,
    (k + 0.5)/n, first and each half in particle order (the order the
    corrector's half-cell walk relies on); REF keeps particle order."""
    n = 48
    sc = crowded_scene(n, 4) if crowd else scenes.pool_sphere(n, seed=4)
    for arith in (gpu.ARITH_FAST, gpu.ARITH_REF):
        prm = gpu.default_params(n, sc.count, solve_mode=gpu.SOLVE_FAST,
                                 precond=gpu.PRECOND_MG, arith=arith)
        sim = gpu.Simulation(prm)
        sim.set_particles(sc.pos, sc.type, sc.vel, sc.nrm)
        sim.sort()
        cs, perm = sim.get_cells()
        sim.close()
        z = sc.pos[:, 2]
        k = np.clip((z * np.float32(n)).astype(np.int64), 0, n - 1)
        mid = ((k.astype(np.float32) + np.float32(0.5)) * np.float32(1.0 / n)).astype(np.float32)
        up = (z >= mid).astype(np.int64)
        cell = np.repeat(np.arange(n ** 3), np.diff(cs.astype(np.int64)))
        key = (cell << 33) + ((up[perm] << 32) if arith == gpu.ARITH_FAST else 0) + perm
        assert np.all(np.diff(key) > 0), arith


def test_switching_arithmetic_sorts_again(gpu):
    """Lists sorted under FAST arithmetic (lower z half first) are not used
    by REF gathers after flipgpu_set_params switches to REF: the density
    then equals a REF handle's bit for bit."""
    n = 40
    sc = scenes.pool_sphere(n, seed=6)
    out = {}
    for first in (gpu.ARITH_FAST, gpu.ARITH_REF):
        prm = gpu.default_params(n, sc.count, arith=first)
        sim = gpu.Simulation(prm)
        sim.set_particles(sc.pos, sc.type, sc.vel, sc.nrm)
        sim.set_max_density(25.0)
        sim.sort()
        sim.set_params(gpu.default_params(n, sc.count, arith=gpu.ARITH_REF))
        sim.compute_density()
        out[first] = sim.get_particles()[2]
        sim.close()
    assert np.array_equal(out[gpu.ARITH_FAST], out[gpu.ARITH_REF])

"""MG-preconditioned CG (FLIPGPU_PRECOND_MG) against FP64 solves of the same
systems on the oracle, on grids whose level hierarchies differ: 16 and 32
(every coarse level inside one block), 48 (odd coarse sizes 3..24), 64 (a
grid-wide middle level)."""
import numpy as np
import pytest

from flip3d_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from flip3d_gb300 import gpu as g
    g.load()
    return g


@pytest.fixture(scope="module")
def orc():
    from oracle import pyoracle
    return pyoracle


def system(orc, n, seed=1, scene="dam_break"):
    sc = getattr(scenes, scene)(n, seed=seed)
    cs, perm = orc.sort(n, sc.pos)
    dens = orc.density(n, sc.pos, sc.type, cs, perm, orc.max_density(n))
    A = orc.mark_water(n, sc.type, dens, cs, perm)
    L = orc.levelset(n, sc.type, dens, cs, perm)
    b = np.where(A == 1, np.random.default_rng(seed).normal(0, 1, n ** 3), 0).astype(np.float32)
    return A, L, b


def fast_solve(gpu, n, A, L, b, precond):
    sim = gpu.Simulation(gpu.default_params(n, 1, rel_tol=1e-6, solve_mode=gpu.SOLVE_FAST,
                                            precond=precond))
    sim.set_grid(A=A, L=L, press=np.zeros(n ** 3, np.float32), div=b)
    st = sim.solve()
    st.x64 = sim.get_pressure()
    return st, sim.get_grid()[3]


@pytest.mark.parametrize("n,scene", [(16, "dam_break"), (32, "pool_sphere"), (48, "dam_break"),
                                     (64, "dam_break")])
def test_mg_pcg_solves_the_system(gpu, orc, n, scene):
    A, L, b = system(orc, n, scene=scene)
    st, p = fast_solve(gpu, n, A, L, b, gpu.PRECOND_MG)
    assert st.status == 0
    assert st.r2 <= 1e-12 * st.b2 * (1 + 1e-9)
    # the true residual of the refined iterate, in FP64 on the host
    r = orc.fast_residual_fp64(n, A, L, -b, st.x64)
    fl = A == 1
    assert np.linalg.norm(r[fl]) <= 1e-6 * np.linalg.norm(b[fl].astype(np.float64))
    st_j, _ = fast_solve(gpu, n, A, L, b, gpu.PRECOND_JACOBI)
    # a V-cycle per iteration: a few times fewer iterations than Jacobi
    # (refinement passes of both summed)
    assert st.iterations <= 40 and st.iterations * 3 < st_j.iterations, (st.iterations,
                                                                         st_j.iterations)
    x, _, _, _, _ = orc.solve(orc.params(n, orc.PRECOND_IC, rel_tol=1e-12), A, L,
                              np.zeros(n ** 3, np.float32), b)
    fl = A == 1
    err = np.linalg.norm((p - x)[fl]) / np.linalg.norm(x[fl])
    assert err < 1e-3, err


def test_mg_pcg_at_full_size(gpu, orc):
    """The N=128 dam break (every SM in the grid, four grid-wide levels):
    iteration count, the true residual of the refined iterate in FP64 on the
    host (<= 1e-6 of ||b||), and two solves bit-identical (a race between the
    phases would break that)."""
    n = 128
    A, L, b = system(orc, n)
    sols = []
    for _ in range(2):
        sim = gpu.Simulation(gpu.default_params(n, 1, rel_tol=1e-6, solve_mode=gpu.SOLVE_FAST,
                                                precond=gpu.PRECOND_MG, max_iters=200))
        sim.set_grid(A=A, L=L, press=np.zeros(n ** 3, np.float32), div=b)
        st = sim.solve()
        assert st.status == 0 and st.iterations <= 60, (st.status, st.iterations)
        sols.append(sim.get_pressure())
    diff = int(np.sum(sols[0] != sols[1]))
    assert diff == 0, f"{diff} values differ between two solves"
    # the solver answers A x = -b (the reference negates b, src/solver.cpp:231)
    r = orc.fast_residual_fp64(n, A, L, -b, sols[0])
    fl = A == 1
    rel = np.linalg.norm(r[fl]) / np.linalg.norm(b[fl].astype(np.float64))
    assert rel <= 1e-6, rel


def test_mg_pcg_is_deterministic(gpu, orc):
    A, L, b = system(orc, 32)
    st1, p1 = fast_solve(gpu, 32, A, L, b, gpu.PRECOND_MG)
    st2, p2 = fast_solve(gpu, 32, A, L, b, gpu.PRECOND_MG)
    assert st1.iterations == st2.iterations
    assert np.array_equal(p1, p2)


def test_mg_steps_track_jacobi_steps(gpu, orc):
    """Three simulation steps with the MG-preconditioned solve agree with
    the Jacobi-preconditioned ones to the solver tolerance."""
    sc = scenes.dam_break(48, seed=2)
    md = orc.max_density(48)
    sims = []
    for pre in (gpu.PRECOND_JACOBI, gpu.PRECOND_MG):
        s = gpu.Simulation(gpu.default_params(48, sc.count, rel_tol=1e-6, seed=3,
                                              solve_mode=gpu.SOLVE_FAST, precond=pre))
        s.set_scene(sc)
        s.set_max_density(md)
        sims.append(s)
    for _ in range(3):
        for s in sims:
            assert s.step().status == 0
    (pj, vj, _, tj), (pm, vm, _, _) = sims[0].get_particles(), sims[1].get_particles()
    fl = tj == 1
    assert np.abs(pj - pm).max() <= 2e-5
    assert np.abs(vj[fl] - vm[fl]).max() <= 2e-3 * max(float(np.abs(vj[fl]).max()), 1.0)


def test_mg_needs_quads(gpu, orc):
    A, L, b = system(orc, 13)
    sim = gpu.Simulation(gpu.default_params(13, 1, rel_tol=1e-6, solve_mode=gpu.SOLVE_FAST,
                                            precond=gpu.PRECOND_MG))
    sim.set_grid(A=A, L=L, press=np.zeros(13 ** 3, np.float32), div=b)
    with pytest.raises(gpu.FlipGpuError):
        sim.solve()

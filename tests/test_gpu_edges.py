"""Edge cases of the step and its side paths: no particles at all, walls
and no liquid, a ragged grid (n = 17, not a multiple of the 4-cell quads
or the 16-cell bricks) against the oracle, and the argument and capacity
errors of the C ABI."""
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


def _fast(gpu, n, cap, **kw):
    return gpu.Simulation(gpu.default_params(n, cap, rel_tol=1e-6, solve_mode=gpu.SOLVE_FAST,
                                             precond=gpu.PRECOND_JACOBI, **kw))


def test_no_particles(gpu, tmp_path):
    sim = _fast(gpu, 16, 64)
    sim.set_particles(np.zeros((0, 3), np.float32), np.zeros(0, np.uint8))
    for _ in range(2):
        st = sim.step()
        assert st.status == 0 and st.iterations == 0
    pos, vel, dens, typ = sim.get_particles()
    assert pos.shape == (0, 3)
    m = sim.mesh()
    assert m["vertices"].shape[0] == 0 and m["faces"].shape[0] == 0
    img = sim.preview(64, 48)
    assert (img[..., :3] == 0).all() and (img[..., 3] == 255).all()
    path = str(tmp_path / "empty.dat")
    sim.save_state(path)
    assert gpu.checkpoint_read(path, 16)["count"] == 0


@pytest.mark.parametrize("precond", ["jacobi", "mic"])
def test_walls_without_liquid(gpu, tmp_path, precond):
    n = 16
    sim = gpu.Simulation(gpu.default_params(
        n, 4096, rel_tol=1e-6, solve_mode=gpu.SOLVE_FAST,
        precond=gpu.PRECOND_JACOBI if precond == "jacobi" else gpu.PRECOND_IC,
        mic_tau=0.97 if precond == "mic" else 0.0))
    sim.seed_scene([], seed=0)
    assert sim.np == n ** 3 - (n - 2) ** 3
    sim.calibrate_max_density()
    before = sim.get_particles()
    for _ in range(2):
        st = sim.step()
        assert st.status == 0
    after = sim.get_particles()
    assert np.array_equal(before[0], after[0])  # walls never move
    _, A, _, press, _ = sim.get_grid()
    assert not (A == 1).any() and not press.any()
    assert sim.mesh()["faces"].shape[0] == 0
    path = str(tmp_path / "walls.dat")
    sim.save_state(path)
    other = gpu.Simulation(gpu.default_params(n, 4096))
    other.load_state(path)
    for x, y in zip(sim.get_particles(), other.get_particles()):
        assert np.array_equal(x, y)


def test_ragged_grid_matches_the_oracle(gpu, orc):
    """n = 17: the REF step against the oracle, and the FAST step (scalar
    CG path, partial wavefront bricks) to the FAST-step tolerance."""
    sc = scenes.pool_sphere(17, seed=3)
    n = sc.n
    md = orc.max_density(n)
    osim = orc.Sim(sc, orc.params(n, orc.PRECOND_REF, rel_tol=1e-6, seed=4), md)
    ref = gpu.Simulation(gpu.default_params(n, sc.count, rel_tol=1e-6, seed=4))
    fast = _fast(gpu, n, sc.count, seed=4, arith=gpu.ARITH_FAST)
    mic = gpu.Simulation(gpu.default_params(n, sc.count, rel_tol=1e-6, seed=4,
                                            solve_mode=gpu.SOLVE_FAST, precond=gpu.PRECOND_IC,
                                            mic_tau=0.97))
    for s in (ref, fast, mic):
        s.set_scene(sc)
        s.set_max_density(md)
    for _ in range(2):
        osim.step()
        for s in (ref, fast, mic):
            assert s.step().status == 0
    opos, ovel, _, otyp = osim.get()
    fl = otyp == 1
    vscale = max(float(np.abs(ovel[fl]).max()), 1.0)
    rp = ref.get_particles()
    assert np.abs(rp[0] - opos).max() <= 1e-5
    for s in (fast, mic):
        p = s.get_particles()
        assert np.abs(p[0] - opos).max() <= 2e-5
        assert np.abs(p[1][fl] - ovel[fl]).max() <= 2e-3 * vscale


def test_errors_are_reported(gpu, tmp_path):
    sim = _fast(gpu, 16, 100)
    with pytest.raises(gpu.FlipGpuError):
        sim.set_particles(np.zeros((200, 3), np.float32), np.ones(200, np.uint8))
    with pytest.raises(gpu.FlipGpuError):
        sim.load_state(str(tmp_path / "missing.dat"))
    with pytest.raises(gpu.FlipGpuError):
        sim.seed_scene([scenes.Box((0.1, 0.1, 0.1), (0.9, 0.9, 0.9))] * 17, 0)
    with pytest.raises(gpu.FlipGpuError):
        gpu.Simulation(gpu.default_params(2, 10))

"""CUDA path (through the C ABI) against the CPU oracle on the same inputs.

The oracle is pinned bit-exact to the reference (test_oracle_golden.py), so
equality here is equality with the reference. Integer and index results must
match exactly; float results of every stage are expected to match bit for bit
(the kernels follow the reference's evaluation order and promotions), with
one stated exception: the FP64 dot products of the solver are summed as a
tree instead of sequentially, which can move the CG scalars by ~1e-16 and a
pressure value by an ulp. Those comparisons carry an explicit tolerance.
"""
import numpy as np
import pytest

from flip3d_gb300 import scenes

pytestmark = pytest.mark.gpu

GOLD = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def gpu():
    from flip3d_gb300 import gpu as g
    g.load()
    return g


@pytest.fixture(scope="module")
def orc():
    from oracle import pyoracle
    return pyoracle


def make_sim(gpu, n, np_, **kw):
    p = gpu.default_params(n, max(np_, 1), **kw)
    return gpu.Simulation(p)


def comp_inputs(name):
    g = np.load(f"{GOLD}/{name}.npz")
    return g


@pytest.mark.parametrize("name", ["components_n16", "components_n13"])
def test_sort_matches_reference(gpu, name):
    g = comp_inputs(name)
    n = int(g["n"])
    sim = make_sim(gpu, n, g["pos"].shape[0])
    sim.set_particles(g["pos"], g["type"], g["vel"], g["nrm"], g["dens"])
    sim.sort()
    cs, perm = sim.get_cells()
    assert np.array_equal(cs, g["cell_start"])
    assert np.array_equal(perm, g["perm"])


@pytest.mark.parametrize("name", ["components_n16", "components_n13"])
def test_mark_water_matches_reference(gpu, name):
    g = comp_inputs(name)
    n = int(g["n"])
    sim = make_sim(gpu, n, g["pos"].shape[0])
    sim.set_particles(g["pos"], g["type"], g["vel"], g["nrm"], g["dens"])
    sim.sort()
    sim.mark_water()
    _, A, L, _, _ = sim.get_grid()
    assert np.array_equal(A, g["A"])
    assert np.array_equal(L, g["L"])


@pytest.mark.parametrize("name", ["components_n16", "components_n13"])
def test_p2g_matches_reference(gpu, name):
    g = comp_inputs(name)
    n = int(g["n"])
    sim = make_sim(gpu, n, g["pos"].shape[0])
    sim.set_particles(g["pos"], g["type"], g["vel"], g["nrm"])
    sim.sort()
    sim.p2g()
    u, _, _, _, _ = sim.get_grid()
    for c in range(3):
        assert np.array_equal(u[c], g[f"u{c}"]), f"component {c}"


@pytest.mark.parametrize("name", ["components_n16", "components_n13"])
def test_g2p_matches_reference(gpu, orc, name):
    g = comp_inputs(name)
    n = int(g["n"])
    sim = make_sim(gpu, n, g["pos"].shape[0])
    sim.set_particles(g["pos"], g["type"], g["vel"], g["nrm"])
    grid = [g["grid0"], g["grid1"], g["grid2"]]
    sim.set_grid(u=grid)
    sim.g2p()
    _, vel, _, _ = sim.get_particles()
    ref = orc.g2p(n, g["pos"], g["type"], grid)
    assert np.array_equal(vel, ref)
    # every particle, walls included, where the reference stays inside its
    # arrays (n*z > n-0.5 reads past a row of the v grid in the reference)
    ub = (np.float32(n) * g["pos"][:, 2]) > np.float32(n - 0.5)
    assert np.array_equal(vel[~ub], g["g2p"][~ub])


@pytest.mark.parametrize("name", ["components_n16", "components_n13"])
def test_point_queries_match_oracle(gpu, orc, name):
    """mapper::fetchVelocity and corrector::resample at arbitrary points."""
    g = comp_inputs(name)
    n = int(g["n"])
    sim = make_sim(gpu, n, g["pos"].shape[0])
    sim.set_particles(g["pos"], g["type"], g["vel"], g["nrm"])
    grid = [g["grid0"], g["grid1"], g["grid2"]]
    sim.set_grid(u=grid)
    rng = np.random.default_rng(5)
    pts = rng.uniform(-0.1, 1.1, (200, 3)).astype(np.float32)
    got = sim.fetch_velocity(pts)
    assert np.array_equal(got, orc.g2p(n, pts, np.ones(200, np.uint8), grid))
    sim.sort()
    cs, perm = sim.get_cells()
    fallback = rng.normal(0, 1, (200, 3)).astype(np.float32)
    for re in (0.5 / n, 1.0 / n):
        got = sim.resample(pts, fallback, re)
        want = np.stack([orc.resample(n, g["pos"], g["vel"], g["type"], cs, perm, pts[t],
                                      fallback[t], re) for t in range(200)])
        assert np.array_equal(got, want)


@pytest.mark.parametrize("name", ["components_n16", "components_n13"])
def test_correct_matches_reference(gpu, name):
    g = comp_inputs(name)
    n = int(g["n"])
    sim = make_sim(gpu, n, g["pos"].shape[0], seed=int(g["corr_seed"]))
    sim.set_particles(g["pos"], g["type"], g["vel"], g["nrm"])
    sim.set_step(int(g["corr_step"]))
    sim.correct()
    pos, vel, _, _ = sim.get_particles()
    fl = g["type"] == 1
    assert np.array_equal(pos, g["corr_pos"])
    assert np.array_equal(vel[fl], g["corr_vel"][fl])


def test_density_matches_oracle(gpu, orc):
    sc = scenes.pool_sphere(32, seed=3)
    n = sc.n
    md = orc.max_density(n)
    sim = make_sim(gpu, n, sc.count)
    sim.set_scene(sc)
    assert np.float32(sim.calibrate_max_density()) == np.float32(md)
    sim.compute_density()
    _, _, dens, _ = sim.get_particles()
    cs, perm = orc.sort(n, sc.pos)
    ref = orc.density(n, sc.pos, sc.type, cs, perm, md)
    assert np.array_equal(dens, ref)


@pytest.mark.parametrize("name", ["solver_n16", "solver_n13"])
@pytest.mark.parametrize("tag,rel", [("abs", 0.0), ("rel6", 1e-6)])
def test_solve_ref_mode_matches_reference(gpu, name, tag, rel):
    """REF-mode PCG against the reference's own solve. Iteration counts equal;
    pressures equal up to the dot-product summation order (|dp| <= 1e-5 of
    max|p|, and in practice almost all values bit-identical)."""
    g = np.load(f"{GOLD}/{name}.npz")
    n = int(g["n"])
    sim = make_sim(gpu, n, 1, rel_tol=rel)
    sim.set_grid(A=g["A"], L=g["L"], press=g["x0"], div=g["b"])
    st = sim.solve()
    _, _, _, p, b = sim.get_grid()
    ref = g[f"x_{tag}"]
    assert np.array_equal(b, g[f"b_{tag}"])
    scale = float(np.abs(ref).max())
    assert np.abs(p - ref).max() <= 1e-5 * scale
    assert np.mean(p == ref) > 0.9


@pytest.mark.parametrize("name", ["solver_n16", "solver_n13"])
def test_solve_fast_mode_converges_to_fp64(gpu, orc, name):
    """FAST mode (FP32 matvec and Jacobi, double-float dot products) to
    rel-res 1e-6 against an FP64 IC(0) solve run to 1e-12 on the oracle.
    n=16 runs the quad-vectorised kernel, n=13 the per-cell one."""
    g = np.load(f"{GOLD}/{name}.npz")
    n = int(g["n"])
    sim = make_sim(gpu, n, 1, rel_tol=1e-6, solve_mode=gpu.SOLVE_FAST,
                   precond=gpu.PRECOND_JACOBI)
    sim.set_grid(A=g["A"], L=g["L"], press=np.zeros(n ** 3, np.float32), div=g["b"])
    st = sim.solve()
    assert st.status == 0
    assert st.r2 <= 1e-12 * st.b2 * (1 + 1e-9)
    _, _, _, p, _ = sim.get_grid()
    prm = orc.params(n, orc.PRECOND_IC, rel_tol=1e-12)
    x, _, it, _, _ = orc.solve(prm, g["A"], g["L"], np.zeros(n ** 3, np.float32), g["b"])
    fl = g["A"] == 1
    err = np.linalg.norm((p - x)[fl]) / np.linalg.norm(x[fl])
    assert err < 1e-4, err


def run_steps_both(gpu, orc, sc, steps, rel_tol, seed=11):
    n = sc.n
    md = orc.max_density(n)
    prm = orc.params(n, orc.PRECOND_REF, rel_tol=rel_tol, seed=seed)
    osim = orc.Sim(sc, prm, md)
    gsim = make_sim(gpu, n, sc.count, rel_tol=rel_tol, seed=seed)
    gsim.set_scene(sc)
    gsim.set_max_density(md)
    for _ in range(steps):
        osim.step()
        gsim.step()
    return osim, gsim


@pytest.mark.parametrize("steps", [1, 3])
def test_full_step_matches_oracle(gpu, orc, steps):
    """simulateStep at N=32 on the pool+sphere scene, rel-res 1e-6."""
    sc = scenes.pool_sphere(32, seed=0)
    osim, gsim = run_steps_both(gpu, orc, sc, steps, 1e-6)
    opos, ovel, odens, otyp = osim.get()
    gpos, gvel, gdens, gtyp = gsim.get_particles()
    fl = otyp == 1
    assert np.array_equal(gtyp, otyp)
    dpos = np.abs(gpos - opos).max()
    dvel = np.abs(gvel[fl] - ovel[fl]).max()
    assert dpos <= 1e-5, dpos
    assert dvel <= 1e-3 * max(1.0, float(np.abs(ovel[fl]).max())), dvel
    assert np.abs(gdens - odens).max() <= 1e-4
    # and most values identical
    assert np.mean(gpos == opos) > 0.95


def test_step_deterministic(gpu):
    sc = scenes.pool_sphere(24, seed=5)
    outs = []
    for _ in range(2):
        sim = make_sim(gpu, sc.n, sc.count, rel_tol=1e-6, seed=2)
        sim.set_scene(sc)
        sim.calibrate_max_density()
        for _ in range(3):
            sim.step()
        outs.append(sim.get_particles())
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)


def test_fast_step_close_to_reference_step(gpu, orc):
    """One FAST-mode step (Jacobi PCG to rel-res 1e-6, FP32) against the
    reference step on the oracle: both solves meet the same relative residual,
    so particle states agree to the solver tolerance."""
    sc = scenes.dam_break(32, seed=2)
    n = sc.n
    md = orc.max_density(n)
    osim = orc.Sim(sc, orc.params(n, orc.PRECOND_REF, rel_tol=1e-6, seed=4), md)
    gsim = make_sim(gpu, n, sc.count, rel_tol=1e-6, seed=4, solve_mode=gpu.SOLVE_FAST,
                    precond=gpu.PRECOND_JACOBI)
    gsim.set_scene(sc)
    gsim.set_max_density(md)
    for _ in range(2):
        osim.step()
        st = gsim.step()
        assert st.status == 0
    opos, ovel, _, otyp = osim.get()
    gpos, gvel, _, _ = gsim.get_particles()
    fl = otyp == 1
    vscale = float(np.abs(ovel[fl]).max())
    print("fast vs ref: max dpos", np.abs(gpos - opos).max(), "max dvel",
          np.abs(gvel[fl] - ovel[fl]).max(), "vscale", vscale)
    assert np.abs(gpos - opos).max() <= 2e-5
    assert np.abs(gvel[fl] - ovel[fl]).max() <= 2e-3 * max(vscale, 1.0)


@pytest.mark.parametrize("tau", [0.0, 0.97])
@pytest.mark.parametrize("name", ["solver_n16", "solver_n13"])
def test_solve_ic_wavefront_matches_fp64_factor(gpu, orc, name, tau):
    """IC(0) (tau=0) / MIC(0) (tau=0.97) applied as brick wavefronts in FP32
    against the oracle's sequential FP64 factor: same solution to rel-res
    1e-6, and iteration counts within 15% of the FP64 run (a wrong factor or
    sweep order shows up as a different count or no convergence)."""
    g = np.load(f"{GOLD}/{name}.npz")
    n = int(g["n"])
    # one PCG (no refinement passes), so that iteration counts compare
    sim = make_sim(gpu, n, 1, rel_tol=1e-6, solve_mode=gpu.SOLVE_FAST,
                   precond=gpu.PRECOND_IC, mic_tau=tau, refine_steps=0)
    sim.set_grid(A=g["A"], L=g["L"], press=np.zeros(n ** 3, np.float32), div=g["b"])
    st = sim.solve()
    assert st.status == 0
    assert st.r2 <= 1e-12 * st.b2 * (1 + 1e-9)
    _, _, _, p, _ = sim.get_grid()
    prm = orc.params(n, orc.PRECOND_IC, rel_tol=1e-6, mic_tau=tau)
    x6, _, it6, _, _ = orc.solve(prm, g["A"], g["L"], np.zeros(n ** 3, np.float32), g["b"])
    prm = orc.params(n, orc.PRECOND_IC, rel_tol=1e-12, mic_tau=tau)
    x, _, _, _, _ = orc.solve(prm, g["A"], g["L"], np.zeros(n ** 3, np.float32), g["b"])
    fl = g["A"] == 1
    err = np.linalg.norm((p - x)[fl]) / np.linalg.norm(x[fl])
    assert err < 1e-4, err
    assert abs(st.iterations - it6) <= max(2, 0.15 * it6), (st.iterations, it6)


def test_solve_mic_on_a_dam_break(gpu, orc):
    """MIC(0) wavefront on a realistic N=32 system (several bricks per axis)."""
    sc = scenes.dam_break(32, seed=1)
    n = sc.n
    cs, perm = orc.sort(n, sc.pos)
    dens = orc.density(n, sc.pos, sc.type, cs, perm, orc.max_density(n))
    A = orc.mark_water(n, sc.type, dens, cs, perm)
    L = orc.levelset(n, sc.type, dens, cs, perm)
    b = np.where(A == 1, np.random.default_rng(1).normal(0, 1, n ** 3), 0).astype(np.float32)
    prm = orc.params(n, orc.PRECOND_IC, rel_tol=1e-6, mic_tau=0.97)
    x6, _, it6, _, _ = orc.solve(prm, A, L, np.zeros(n ** 3, np.float32), b)
    sim = make_sim(gpu, n, 1, rel_tol=1e-6, solve_mode=gpu.SOLVE_FAST,
                   precond=gpu.PRECOND_IC, mic_tau=0.97, refine_steps=0)
    sim.set_grid(A=A, L=L, press=np.zeros(n ** 3, np.float32), div=b)
    st = sim.solve()
    assert st.status == 0
    _, _, _, p, _ = sim.get_grid()
    fl = A == 1
    assert np.linalg.norm((p - x6)[fl]) / np.linalg.norm(x6[fl]) < 1e-4
    assert abs(st.iterations - it6) <= max(2, 0.15 * it6), (st.iterations, it6)


def _forced_reposition_state(orc, sc, seed, wide=False):
    """A state where the fluid particles of one wall slab are stuck. Narrow:
    the only deep-water cell is the centre of a 3^3 fluid block, so every
    stuck particle is re-seeded into the same cell and each resamples next to
    all earlier ones (past the parallel rounds into the ordered tail). Wide:
    the rest of the box is fluid, so the stuck particles fill the first deep
    cells one per cell, a compact block where neighbours depend on each
    other in random order (the parallel rounds)."""
    n = sc.n
    prm = orc.params(n, orc.PRECOND_REF, rel_tol=1e-6, seed=seed)
    o = orc.Sim(sc, prm)
    o.set_step(5)
    o.stage(0)
    A = np.zeros((n, n, n), np.uint8)
    A[0], A[-1], A[:, 0], A[:, -1], A[:, :, 0], A[:, :, -1] = 2, 2, 2, 2, 2, 2
    A[5, 1:5, 1:n - 1] = 2
    if wide:
        A[1:5, 1:n - 1, 1:n - 1] = 1
        A[6:n - 1, 1:n - 1, 1:n - 1] = 1
        A[5, 5:n - 1, 1:n - 1] = 1
    else:
        A[10:13, 2:5, 6:9] = 1
    rng = np.random.default_rng(seed)
    pos, vel, dens, typ = o.get()
    vel = rng.normal(0.0, 1.0, size=vel.shape).astype(np.float32)
    vel[typ != 1] = 0.0
    nf = (n + 1) * n * n
    u = [np.zeros(nf, np.float32) for _ in range(3)]
    zeros = np.zeros(n ** 3, np.float32)
    o.put(vel=vel)
    o.put_grid(u, A.ravel(), zeros, zeros)
    return o, pos, vel, dens, typ, u, A.ravel(), zeros


@pytest.mark.parametrize("wide", [False, True])
def test_reposition_ordered_resample_matches_oracle(gpu, orc, wide):
    sc = scenes.pool_sphere(16, seed=4)
    o, pos, vel, dens, typ, u, A, zeros = _forced_reposition_state(orc, sc, 7, wide)
    g = make_sim(gpu, sc.n, sc.count, seed=7)
    g.set_particles(pos, typ, vel, sc.nrm, dens)
    g.set_grid(u, A, zeros, zeros, zeros)
    g.set_step(5)
    stuck = g.advect()
    o.stage(3)
    assert stuck == o.stuck == 448
    opos, ovel, _, _ = o.get()
    gpos, gvel, _, _ = g.get_particles()
    assert np.array_equal(gpos, opos)
    fl = typ == 1
    assert np.array_equal(gvel[fl], ovel[fl])


@pytest.mark.parametrize("name", ["mesh_n16", "mesh_n13"])
def test_mesh_matches_reference(gpu, orc, name):
    """mesher::generateMesh and implicit::implicit_func against the
    reference's own output on a scrambled scene (bit for bit)."""
    g = np.load(f"{GOLD}/{name}.npz")
    n = int(g["n"])
    sim = make_sim(gpu, n, g["pos"].shape[0])
    sim.set_particles(g["pos"], g["type"])
    sim.sort()
    assert np.array_equal(sim.implicit(g["pts"]), g["phi"])
    m = sim.mesh(field=True)
    cs, perm = orc.sort(n, g["pos"])
    om = orc.mesh(n, g["pos"], g["type"], cs, perm)
    assert np.array_equal(m["field"], om["phi"])
    assert np.array_equal(m["vertices"].ravel(), g["vertices"])
    assert np.array_equal(m["faces"].ravel(), g["faces"])
    assert np.array_equal(m["normals"].ravel(), g["normals"])


def test_mesh_after_steps_matches_oracle(gpu, orc):
    """The mesh write_mesh exports after a step: the corrector's lists over
    post-correction positions, computed on the GPU state and by the oracle
    on that same state."""
    sc = scenes.pool_sphere(32, seed=0)
    sim = make_sim(gpu, sc.n, sc.count, rel_tol=1e-6, seed=3)
    sim.set_scene(sc)
    sim.calibrate_max_density()
    for _ in range(2):
        sim.step()
    pos, vel, dens, typ = sim.get_particles()
    cs, perm = sim.get_cells()
    m = sim.mesh()
    om = orc.mesh(sc.n, pos, typ, cs, perm)
    assert m["vertices"].shape[0] > 1000
    assert np.array_equal(m["vertices"].ravel(), om["vertices"])
    assert np.array_equal(m["faces"].ravel(), om["faces"])
    assert np.array_equal(m["normals"].ravel(), om["normals"])


def test_mesh_on_stale_lists_matches_oracle(gpu, orc):
    """The reference's sorter keeps particle pointers, so a mesh made after
    particles moved reads new positions through old lists. Particles here
    move up to 1.5 cells (a few far away) after the sort."""
    g = np.load(f"{GOLD}/mesh_n16.npz")
    n = int(g["n"])
    pos, typ = g["pos"], g["type"]
    sim = make_sim(gpu, n, pos.shape[0])
    sim.set_particles(pos, typ)
    sim.sort()
    cs, perm = sim.get_cells()
    rng = np.random.default_rng(11)
    moved = pos.copy()
    fl = typ == 1
    moved[fl] += rng.uniform(-1.5 / n, 1.5 / n, size=(fl.sum(), 3)).astype(np.float32)
    far = rng.choice(np.nonzero(fl)[0], 20, replace=False)
    moved[far] = rng.uniform(0.0, 1.0, size=(20, 3)).astype(np.float32)
    sim.put_state(moved, np.zeros_like(moved))
    pts = g["pts"]
    assert np.array_equal(sim.implicit(pts), orc.implicit(n, moved, typ, cs, perm, pts))
    m = sim.mesh(field=True)
    om = orc.mesh(n, moved, typ, cs, perm)
    assert np.array_equal(m["field"], om["phi"])
    assert np.array_equal(m["vertices"].ravel(), om["vertices"])
    assert np.array_equal(m["faces"].ravel(), om["faces"])
    assert np.array_equal(m["normals"].ravel(), om["normals"])


def test_fast_arithmetic_tracks_the_reference_step(gpu, orc):
    """FLIPGPU_ARITH_FAST (native FP32 gathers) against the reference's
    steps on the oracle, 2 steps of the N=32 dam break with the FAST solver:
    the same tolerances as the FAST-solver step test (positions 2e-5 of the
    unit cube, velocities 2e-3 of the largest speed). FAST arithmetic is
    deterministic run to run."""
    sc = scenes.dam_break(32, seed=2)
    n = sc.n
    md = orc.max_density(n)
    osim = orc.Sim(sc, orc.params(n, orc.PRECOND_REF, rel_tol=1e-6, seed=4), md)
    sims = []
    for _ in range(2):
        g = make_sim(gpu, n, sc.count, rel_tol=1e-6, seed=4, solve_mode=gpu.SOLVE_FAST,
                     precond=gpu.PRECOND_JACOBI, arith=gpu.ARITH_FAST)
        g.set_scene(sc)
        g.set_max_density(md)
        sims.append(g)
    for _ in range(2):
        osim.step()
        for g in sims:
            assert g.step().status == 0
    opos, ovel, odens, otyp = osim.get()
    gpos, gvel, gdens, _ = sims[0].get_particles()
    fl = otyp == 1
    vscale = float(np.abs(ovel[fl]).max())
    print("fast arithmetic vs ref: max dpos", np.abs(gpos - opos).max(), "max dvel",
          np.abs(gvel[fl] - ovel[fl]).max(), "max ddens", np.abs(gdens - odens).max())
    assert np.abs(gpos - opos).max() <= 2e-5
    assert np.abs(gvel[fl] - ovel[fl]).max() <= 2e-3 * max(vscale, 1.0)
    assert np.abs(gdens - odens).max() <= 1e-4
    for x, y in zip(sims[0].get_particles(), sims[1].get_particles()):
        assert np.array_equal(x, y)


def _fast_sim(gpu, sc, seed=3, precond=None, arith=None):
    s = make_sim(gpu, sc.n, sc.count, rel_tol=1e-6, seed=seed, solve_mode=gpu.SOLVE_FAST,
                 precond=gpu.PRECOND_JACOBI if precond is None else precond,
                 arith=gpu.ARITH_REF if arith is None else arith)
    s.set_scene(sc)
    s.calibrate_max_density()
    return s


@pytest.mark.parametrize("precond", ["jacobi", "mg", "ic"])
def test_async_and_graph_steps_match_plain_steps(gpu, precond):
    """flipgpu_step_async and a captured CUDA graph replay compute exactly
    what flipgpu_step computes (the device step counter keys the draws),
    with the Jacobi, the multigrid and the IC(0) wavefront persistent solves
    (the graph is captured before any solve ran, so nothing may allocate
    inside it; the wavefront's word tags come from a counter on the device,
    so replays of the same launches never reuse a tag)."""
    sc = scenes.dam_break(32, seed=4)
    pre = {"jacobi": gpu.PRECOND_JACOBI, "mg": gpu.PRECOND_MG, "ic": gpu.PRECOND_IC}[precond]
    ref, asy, gra = (_fast_sim(gpu, sc, precond=pre), _fast_sim(gpu, sc, precond=pre),
                     _fast_sim(gpu, sc, precond=pre))
    gra.capture_step()
    for _ in range(4):
        st = ref.step()
        asy.step_async()
        gra.step_graph()
    a = asy.last_solve_stats()
    g = gra.last_solve_stats()
    assert a.iterations == g.iterations == st.iterations
    for x, y, z in zip(ref.get_particles(), asy.get_particles(), gra.get_particles()):
        assert np.array_equal(x, y) and np.array_equal(x, z)


def test_batch_of_uneven_scenes_matches_one_at_a_time(gpu):
    scs = [scenes.batch_scene(s) for s in (1, 2, 3, 4)]
    assert len({sc.n for sc in scs}) > 1
    alone = [_fast_sim(gpu, sc, seed=i) for i, sc in enumerate(scs)]
    batched = [_fast_sim(gpu, sc, seed=i) for i, sc in enumerate(scs)]
    b = gpu.Batch(batched)
    b.capture()
    for _ in range(3):
        for s in alone:
            s.step()
        b.step()
    b.sync()
    for s, t in zip(alone, batched):
        for x, y in zip(s.get_particles(), t.get_particles()):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("precond", ["jacobi", "mg"])
def test_tuned_batch_matches_lone_handles_with_its_grids(gpu, precond):
    """flipbatch_tune times the members' solves with shared grids and puts
    every member's pressure back: after it, the members hold what one step
    left (the same pressure as lone handles), and stepping on with the tuned
    grids (re-captured graphs) gives the bits of lone handles given the
    same flipgpu_set_solve_blocks."""
    scs = [scenes.batch_scene(s) for s in (5, 6, 7, 8, 9)]
    pc = gpu.PRECOND_MG if precond == "mg" else gpu.PRECOND_JACOBI
    # multigrid wants N a multiple of 4 (every batch_scene size is); it runs
    # with the FAST gathers, as the batch benchmark does
    ar = gpu.ARITH_FAST if precond == "mg" else gpu.ARITH_REF
    alone = [_fast_sim(gpu, sc, seed=i, precond=pc, arith=ar) for i, sc in enumerate(scs)]
    batched = [_fast_sim(gpu, sc, seed=i, precond=pc, arith=ar) for i, sc in enumerate(scs)]
    b = gpu.Batch(batched)
    b.capture()
    for s in alone:
        s.step()
    b.step()
    b.sync()
    share = b.tune()
    caps = [t.solve_blocks() for t in batched]
    print(f"{precond}: share {share}, grids {caps}\n{gpu.autotune_report()}")
    assert share in (0.0, 0.5, 1.0, 2.0, 4.0, 8.0, 16.0)
    assert (share == 0.0) == all(c == 0 for c in caps)
    for s, t in zip(alone, batched):
        assert np.array_equal(s.get_pressure(), t.get_pressure())
        s.solve_blocks(t.solve_blocks())
    for _ in range(3):
        for s in alone:
            assert s.step().status == 0
        b.step()
    b.sync()
    for s, t in zip(alone, batched):
        assert t.last_solve_stats().status == 0
        for x, y in zip(s.get_particles(), t.get_particles()):
            assert np.array_equal(x, y)


def test_batch_tune_needs_a_step_and_leaves_the_wavefront_uncapped(gpu):
    """flipbatch_tune refuses a batch whose members have not stepped; in a
    batch that mixes a multigrid member with an IC(0) wavefront member (which
    keeps its full grid) it caps only the former, and both then step as lone
    handles with the same caps do."""
    scs = [scenes.batch_scene(s) for s in (11, 12)]
    pcs = [gpu.PRECOND_MG, gpu.PRECOND_IC]
    mk = lambda: [_fast_sim(gpu, sc, seed=i, precond=pc, arith=gpu.ARITH_FAST)
                  for i, (sc, pc) in enumerate(zip(scs, pcs))]
    alone, batched = mk(), mk()
    b = gpu.Batch(batched)
    with pytest.raises(gpu.FlipGpuError):
        b.tune()
    for s in alone:
        assert s.step().status == 0
    b.step()
    b.sync()
    share = b.tune()
    caps = [t.solve_blocks() for t in batched]
    print(f"share {share}, grids {caps}")
    assert caps[1] == 0
    assert (share == 0.0) == (caps[0] == 0)
    for s, t in zip(alone, batched):
        s.solve_blocks(t.solve_blocks())
    for _ in range(2):
        for s in alone:
            assert s.step().status == 0
        b.step()
    b.sync()
    for s, t in zip(alone, batched):
        assert t.last_solve_stats().status == 0
        for x, y in zip(s.get_particles(), t.get_particles()):
            assert np.array_equal(x, y)


def test_stage_and_kernel_profiles(gpu):
    """The profiling mode's stage times and its per-kernel times (CUDA events
    around the main kernels' launches) cover the step: one launch of each
    FAST gather per step, the refined multigrid solve's launches, and kernel
    times that fit inside their stages; profiling changes no bit."""
    sc = scenes.dam_break(48, seed=7)
    sims = [_fast_sim(gpu, sc, seed=2, precond=gpu.PRECOND_MG, arith=gpu.ARITH_FAST)
            for _ in range(2)]
    sims[0].set_profiling(True)
    steps = 3
    for _ in range(steps):
        for s in sims:
            assert s.step().status == 0
    stages = sims[0].profile()
    kern = sims[0].kernel_profile()
    sims[0].set_profiling(False)
    print(stages, kern)
    for k in ("k_density", "k_p2g_cells", "k_spring_inline", "k_resample_inline",
              "k_flip_advect"):
        assert kern[k][1] == steps, k
        assert kern[k][0] > 0.0
    assert kern["k_cg_mg"][1] >= steps
    assert kern["k_density"][0] <= stages["density"][0] * 1.001
    assert kern["k_p2g_cells"][0] <= stages["p2g"][0] * 1.001
    assert kern["k_cg_mg"][0] <= stages["solve"][0] * 1.001
    assert (kern["k_spring_inline"][0] + kern["k_resample_inline"][0]
            <= stages["correct"][0] * 1.001)
    for x, y in zip(sims[0].get_particles(), sims[1].get_particles()):
        assert np.array_equal(x, y)
    # switching profiling on again starts from zero
    sims[0].set_profiling(True)
    assert sims[0].kernel_profile() == {}
    sims[0].set_profiling(False)


def test_gather_block_sizes_give_the_same_bits(gpu, monkeypatch):
    """The FAST gathers' block size (tuned per kernel and problem size)
    changes no bit: three steps with 128, 256 and 512 threads per block, and
    with the tuner's own choice, agree."""
    sc = scenes.dam_break(40, seed=2)
    outs = []
    for blk in ("128", "256", "512", ""):
        monkeypatch.setenv("FLIPGPU_GATHER_BLOCK", blk)
        s = _fast_sim(gpu, sc, seed=4, precond=gpu.PRECOND_MG, arith=gpu.ARITH_FAST)
        for _ in range(3):
            assert s.step().status == 0
        outs.append(s.get_particles())
        s.close()
    print(gpu.autotune_report())
    for o in outs[1:]:
        for x, y in zip(outs[0], o):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("fast", [False, True])
def test_step_host_matches_put_step_get(gpu, fast):
    """flipgpu_step_host (transfers overlapped with the step on a second
    stream) gives the same bits as put_state + step + get_particles, with
    the output fed back as the next input."""
    sc = scenes.dam_break(48, seed=5)
    kw = dict(rel_tol=1e-6, seed=6)
    if fast:
        kw.update(solve_mode=gpu.SOLVE_FAST, precond=gpu.PRECOND_MG, arith=gpu.ARITH_FAST)
    sims = [make_sim(gpu, 48, sc.count, **kw) for _ in range(2)]
    for s in sims:
        s.set_scene(sc)
        s.calibrate_max_density()
    pos0, vel0, _, _ = sims[0].get_particles()
    pa, va = pos0.copy(), vel0.copy()
    pb, vb = pos0.copy(), vel0.copy()
    for _ in range(3):
        sims[0].put_state(pa, va)
        assert sims[0].step().status == 0
        pa, va, _, _ = sims[0].get_particles()
        assert sims[1].step_host(pb, vb, pb, vb).status == 0
        assert np.array_equal(pa, pb) and np.array_equal(va, vb)

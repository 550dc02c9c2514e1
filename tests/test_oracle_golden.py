"""The CPU oracle against golden vectors produced by the reference's own C++
(tests/golden/make_golden.py). Everything here is bit-exact except where the
reference reads past an array (see test_g2p)."""
import hashlib

import numpy as np
import pytest

from flip3d_gb300 import scenes
from oracle import pyoracle as orc

GOLD = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load(name):
    return np.load(f"{GOLD}/{name}.npz", allow_pickle=False)


@pytest.fixture(scope="module", params=["components_n16", "components_n13"])
def comp(request):
    g = load(request.param)
    cs, perm = orc.sort(int(g["n"]), g["pos"])
    return g, cs, perm


def test_sort_cell_lists(comp):
    g, cs, perm = comp
    assert np.array_equal(cs, g["cell_start"])
    assert np.array_equal(perm, g["perm"])


def test_mark_water_levelset(comp):
    g, cs, perm = comp
    n = int(g["n"])
    assert np.array_equal(orc.mark_water(n, g["type"], g["dens"], cs, perm), g["A"])
    assert np.array_equal(orc.levelset(n, g["type"], g["dens"], cs, perm), g["L"])


def test_p2g(comp):
    g, cs, perm = comp
    n = int(g["n"])
    u = orc.p2g(n, g["pos"], g["vel"], g["type"], cs, perm)
    for c in range(3):
        assert np.array_equal(u[c], g[f"u{c}"])


def test_g2p(comp):
    """Bit-exact wherever the reference stays inside its arrays. For n*z >
    n-0.5 (outside the walls) the reference's v fetch reads one element past
    a row (src/mapper.cpp:102), which is undefined memory."""
    g, cs, perm = comp
    n = int(g["n"])
    v = orc.g2p(n, g["pos"], g["type"], [g["grid0"], g["grid1"], g["grid2"]])
    ub = (np.float32(n) * g["pos"][:, 2]) > np.float32(n - 0.5)
    assert np.array_equal(v[~ub], g["g2p"][~ub])
    assert np.array_equal(v[ub][:, [0, 2]], g["g2p"][ub][:, [0, 2]])


def test_correct(comp):
    g, cs, perm = comp
    n = int(g["n"])
    p2, v2 = orc.correct(n, g["pos"], g["vel"], g["type"], g["nrm"], cs, perm, 0.006,
                         0.5 / n, int(g["corr_seed"]), int(g["corr_step"]))
    assert np.array_equal(p2, g["corr_pos"])
    assert np.array_equal(v2, g["corr_vel"])


@pytest.mark.parametrize("name", ["solver_n16", "solver_n13"])
@pytest.mark.parametrize("tag,rel", [("abs", 0.0), ("rel6", 1e-6)])
def test_solver(name, tag, rel):
    g = load(name)
    n = int(g["n"])
    prm = orc.params(n, orc.PRECOND_REF, rel_tol=rel)
    x, b, it, r2, b2 = orc.solve(prm, g["A"], g["L"], g["x0"], g["b"])
    assert np.array_equal(x, g[f"x_{tag}"])
    assert np.array_equal(b, g[f"b_{tag}"])


@pytest.mark.parametrize("name", ["driver_n32", "driver_n32_abs"])
def test_driver_steps(name):
    """Whole simulateStep stages at N=32 (src/flip3D.cpp:1194-1264), compared
    stage by stage for step 1 and after steps 2, 5 and 10."""
    g = load(name)
    n = int(g["n"])
    sc = scenes.pool_sphere(n, seed=0)
    assert sha(sc.pos) == str(g["scene_pos_sha"])
    md = orc.max_density(n)
    assert np.float32(md) == g["max_dens"]
    prm = orc.params(n, orc.PRECOND_REF, rel_tol=float(g["rel_tol"]), seed=int(g["seed"]))
    sim = orc.Sim(sc, prm, md)

    def check(tag):
        pos, vel, dens, typ = sim.get()
        u, A, L, pr = sim.grid()
        fl = typ == 1
        for nm, arr in (("pos", pos), ("vel_fluid", np.where(fl[:, None], vel, 0)),
                        ("dens", dens), ("u0", u[0]), ("u1", u[1]), ("u2", u[2]), ("A", A),
                        ("L", L), ("press", pr)):
            assert sha(arr) == str(g[f"{tag}_{nm}_sha"]), f"{tag} {nm}"
        assert sim.stuck == int(g[f"{tag}_stuck"])

    sim.set_step(1)
    for st in range(5):
        sim.stage(st)
        check(f"s1_stage{st}")
    steps = int(g["steps"])
    for k in range(2, steps + 1):
        sim.step()
        if k in (2, 5, steps):
            check(f"step{k}")


@pytest.mark.parametrize("name", ["mesh_n16", "mesh_n13"])
def test_mesh_and_implicit(name):
    """implicit::implicit_func and mesher::generateMesh (field, marching
    cubes, face filter, normals, two smoothing passes) on a scrambled scene."""
    g = load(name)
    n = int(g["n"])
    cs, perm = orc.sort(n, g["pos"])
    phi = orc.implicit(n, g["pos"], g["type"], cs, perm, g["pts"])
    assert np.array_equal(phi, g["phi"])
    m = orc.mesh(n, g["pos"], g["type"], cs, perm)
    for k in ("vertices", "normals", "faces"):
        assert np.array_equal(m[k], g[k]), k


def test_mesh_after_driver_steps():
    """The mesh write_mesh exports after three N=32 steps
    (src/flip3D.cpp:999-1004, 1254-1257): digests of the full arrays."""
    g = load("mesh_driver_n32")
    n = int(g["n"])
    sc = scenes.pool_sphere(n, seed=0)
    md = orc.max_density(n)
    prm = orc.params(n, orc.PRECOND_REF, rel_tol=float(g["rel_tol"]), seed=int(g["seed"]))
    sim = orc.Sim(sc, prm, md)
    for _ in range(int(g["steps"])):
        sim.step()
    m = sim.mesh()
    assert m["vertices"].shape[0] // 3 == int(g["counts"][0])
    assert m["faces"].shape[0] // 3 == int(g["counts"][1])
    assert np.array_equal(m["vertices"][g["vsub"]], g["vertices_sub"])
    assert np.array_equal(m["normals"][g["vsub"]], g["normals_sub"])
    assert np.array_equal(m["faces"][g["fsub"]], g["faces_sub"])
    assert sha(m["vertices"]) == str(g["vertices_sha"])
    assert sha(m["normals"]) == str(g["normals_sha"])
    assert sha(m["faces"]) == str(g["faces_sha"])


def test_fast_operator_restatement_matches_the_oracle_matvec():
    """The FP64 restatement of the FAST-mode operator (fast_residual_fp64,
    used to check refined solves on the host) against the oracle's
    compute_Ax (src/solver.cpp:29-41) on a reference system: the two differ
    only in where float rounding happens."""
    g = np.load(GOLD + "/solver_n16.npz")
    n = int(g["n"])
    A, L = g["A"], g["L"]
    x = np.random.default_rng(3).normal(0, 1, n ** 3).astype(np.float32)
    ax_ref = orc.matvec(n, A, L, x).astype(np.float64)
    ax = -orc.fast_residual_fp64(n, A, L, np.zeros(n ** 3, np.float32), x)
    fl = A == 1
    scale = np.abs(ax_ref[fl]).max()
    assert np.abs(ax[fl] - ax_ref[fl]).max() <= 1e-5 * scale
    assert not ax[~fl].any()

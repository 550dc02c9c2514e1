"""Errors against an FP64 run of the reference: the reference's own sources
built with FLOAT = double (oracle/build_ref64.sh), stepped from the same
seeded scene with the same keyed random draws, recorded by
tests/golden/make_golden.py (tasks fp64_n32, fp64_n128) as particle subsets,
the i = n/4 plane of the pressure and face velocities, and full-set
aggregates.

Two GPU configurations are compared with it:
  ref   the reference's float arithmetic bit for bit (REF solver and
        gathers): its error is the float reference's own error;
  fast  the benchmark's configuration: FAST gathers, multigrid PCG refined
        to a true relative residual of 1e-6.

Stated tolerances (each assert below): per-particle positions and
velocities while the flow is still deterministic at this resolution
(N=32: steps 1 and 10; N=128: steps 1, 5 and 10), pressure and face
velocities on the plane (fluid cells), and the fluid's centre of mass and
kinetic energy at every snapshot, including after 50 and 200 steps at N=32
and 25 and 50 steps at N=128, where individual particles have left the
FP64 trajectories (the flow is chaotic) but the aggregates have not. The
errors are printed."""
import os

import numpy as np
import pytest

from flip3d_gb300 import scenes

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# distances in units of the domain, the rest relative to the FP64 run's
# largest value at that snapshot
TOL = {
    "pos_pp": 1e-4,      # max |dp| per particle, deterministic steps
    "vel_pp": 1e-2,      # max |du| / max |u|, deterministic steps
    "press": 1e-2,       # max |dp| / max |p| on the plane's fluid cells
    "faces": 1e-2,       # max |du_face| / max |u_face| on the plane
    "com": 2e-3,         # |d centre of mass|
    "ke": 5e-2,          # |d KE| / KE
}
DETERMINISTIC = {32: (1, 10), 128: (1, 5, 10)}


@pytest.fixture(scope="module")
def gpu():
    from flip3d_gb300 import gpu as g
    g.load()
    return g


def run(gpu, g, mode):
    n = int(g["n"])
    sc = getattr(scenes, str(g["scene"]))(n, seed=0)
    assert sc.count == int(g["count"])
    kw = dict(rel_tol=1e-6, seed=int(g["seed"]))
    if mode == "fast":
        kw.update(solve_mode=gpu.SOLVE_FAST, precond=gpu.PRECOND_MG, arith=gpu.ARITH_FAST)
    sim = gpu.Simulation(gpu.default_params(n, sc.count, **kw))
    sim.set_scene(sc)
    sim.calibrate_max_density()
    sub = g["subset"]
    fluid = sc.type == 1
    plane_i = int(g["plane"])
    out = {}
    snaps = [int(s) for s in g["snaps"]]
    for k in range(1, max(snaps) + 1):
        st = sim.step()
        assert st.status == 0
        if k in snaps:
            pos, vel, _, _ = sim.get_particles()
            u, A, _, p, _ = sim.get_grid()
            out[k] = {
                "pos": pos[sub].astype(np.float64),
                "vel": np.where(fluid[sub, None], vel[sub], 0.0).astype(np.float64),
                "press": p.reshape(n, n, n)[plane_i].astype(np.float64),
                "u0": u[0].reshape(n + 1, n, n)[plane_i].astype(np.float64),
                "u1": u[1].reshape(n, n + 1, n)[plane_i].astype(np.float64),
                "u2": u[2].reshape(n, n, n + 1)[plane_i].astype(np.float64),
                "com": pos[fluid].astype(np.float64).mean(axis=0),
                "ke": 0.5 * float((vel[fluid].astype(np.float64) ** 2).sum()) / fluid.sum(),
            }
    sim.close()
    return out


def errors(g, k, got):
    t = f"step{k}"
    fl = g[f"{t}_A"] == 1
    assert fl.any(), "the plane holds no liquid"
    e = {"pos_pp": float(np.abs(got["pos"] - g[f"{t}_pos"]).max()),
         "vel_pp": float(np.abs(got["vel"] - g[f"{t}_vel"]).max() /
                         max(np.abs(g[f"{t}_vel"]).max(), 1e-30)),
         "press": float(np.abs(got["press"] - g[f"{t}_press"])[fl].max() /
                        max(np.abs(g[f"{t}_press"][fl]).max(), 1e-30)),
         "com": float(np.abs(got["com"] - g[f"{t}_com"]).max()),
         "ke": abs(got["ke"] - float(g[f"{t}_ke"])) / float(g[f"{t}_ke"])}
    fe = []
    for c in range(3):
        ref = g[f"{t}_u{c}"]
        fe.append(float(np.abs(got[f"u{c}"] - ref).max() / max(np.abs(ref).max(), 1e-30)))
    e["faces"] = max(fe)
    return e


@pytest.mark.parametrize("mode", ["ref", "fast"])
@pytest.mark.parametrize("n", [32, 128])
def test_errors_against_the_fp64_reference(gpu, n, mode):
    g = np.load(os.path.join(GOLD, f"fp64_n{n}.npz"))
    got = run(gpu, g, mode)
    failures = []
    for k in sorted(got):
        e = errors(g, k, got[k])
        print(f"N={n} {mode} step {k}: " + ", ".join(f"{q} {v:.3g}" for q, v in e.items()))
        checks = ["com", "ke"]
        if k in DETERMINISTIC[n]:
            checks += ["pos_pp", "vel_pp", "press", "faces"]
        for q in checks:
            if not e[q] <= TOL[q]:
                failures.append((k, q, e[q], TOL[q]))
    assert not failures, failures

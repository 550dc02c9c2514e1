"""Long-run accuracy statements for the two validation workloads.

  pool:      N=32 pool + sphere, `steps` simulateStep calls (200 by default)
             on the GPU in REF mode (the reference's arithmetic) and by the
             CPU oracle (the reference's algorithm, pinned bit-exact to the
             reference's own build), compared field by field after every
             `every` steps.
  dam_break: N=128 column, the FAST path (FP32 vectors, FP64 dots) against
             the REF path (the reference's solver arithmetic with FP64 dot
             products) from the same state for `steps` steps: the error the
             mixed-precision solver introduces in pressure, velocity and
             position.

    python tests/long_runs.py pool --steps 200
    python tests/long_runs.py dam_break --steps 500
    python tests/long_runs.py dam_break --steps 300 --precond mg --arith fast

Prints one JSON object. Test infrastructure: the oracle is the checker.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from flip3d_gb300 import gpu, scenes  # noqa: E402


def _diff(a, b, mask=None):
    if mask is not None:
        a, b = a[mask], b[mask]
    d = np.abs(a.astype(np.float64) - b.astype(np.float64))
    scale = max(float(np.abs(b).max()), 1e-30)
    return {"max_abs": float(d.max()), "rms": float(np.sqrt((d ** 2).mean())),
            "max_rel_to_max": float(d.max() / scale),
            "identical_frac": float(np.mean(a == b))}


def pool(steps=200, every=20, rel_tol=1e-6, seed=3):
    from oracle import pyoracle as orc
    orc.set_threads(os.cpu_count() or 1)
    sc = scenes.pool_sphere(32, seed=0)
    md = orc.max_density(sc.n)
    osim = orc.Sim(sc, orc.params(sc.n, orc.PRECOND_REF, rel_tol=rel_tol, seed=seed), md)
    g = gpu.Simulation(gpu.default_params(sc.n, sc.count, rel_tol=rel_tol, seed=seed,
                                          solve_mode=gpu.SOLVE_REF, precond=gpu.PRECOND_REF))
    g.set_scene(sc)
    g.calibrate_max_density()
    rec = []
    t0 = time.perf_counter()
    for k in range(1, steps + 1):
        osim.step()
        g.step()
        if k % every == 0 or k == steps:
            opos, ovel, odens, otyp = osim.get()
            gpos, gvel, gdens, gtyp = g.get_particles()
            fl = otyp == 1
            u, A, L, p = osim.grid()
            gu, gA, gL, gp, _ = g.get_grid()
            rec.append({"step": k, "pos": _diff(gpos, opos), "vel_fluid": _diff(gvel, ovel, fl),
                        "press": _diff(gp, p), "A_equal": bool(np.array_equal(gA, A))})
    return {"workload": "pool_sphere N=32, REF mode vs CPU oracle", "steps": steps,
            "rel_tol": rel_tol, "seconds": time.perf_counter() - t0, "records": rec}


def dam_break(steps=500, every=100, rel_tol=1e-6, n=128, precond="jacobi", arith="ref"):
    sc = scenes.dam_break(n, seed=0)
    sims = {}
    fast_pre = gpu.PRECOND_MG if precond == "mg" else gpu.PRECOND_JACOBI
    fast_arith = gpu.ARITH_FAST if arith == "fast" else gpu.ARITH_REF
    for name, mode, pre, ar in (("fast", gpu.SOLVE_FAST, fast_pre, fast_arith),
                                ("ref", gpu.SOLVE_REF, gpu.PRECOND_REF, gpu.ARITH_REF)):
        s = gpu.Simulation(gpu.default_params(n, sc.count, rel_tol=rel_tol, seed=1,
                                              solve_mode=mode, precond=pre, arith=ar))
        s.set_scene(sc)
        s.calibrate_max_density()
        sims[name] = s
    rec = []
    t0 = time.perf_counter()
    for k in range(1, steps + 1):
        for s in sims.values():
            st = s.step()
            if st.status != 0:
                raise RuntimeError(f"step {k}: status {st.status}")
        if k % every == 0 or k == steps or k in (1, 2, 5, 10, 20, 50):
            fp, fv, _, ft = sims["fast"].get_particles()
            rp, rv, _, rt = sims["ref"].get_particles()
            fl = rt == 1
            fgrid, rgrid = sims["fast"].get_grid(), sims["ref"].get_grid()

            def stats(p, v):
                return {"centre": [float(x) for x in p[fl].mean(axis=0)],
                        "mean_speed": float(np.linalg.norm(v[fl], axis=1).mean()),
                        "kinetic": float(0.5 * (v[fl].astype(np.float64) ** 2).sum(axis=1).mean())}
            fs, rs = stats(fp, fv), stats(rp, rv)
            rec.append({"step": k, "pos": _diff(fp, rp), "vel_fluid": _diff(fv, rv, fl),
                        "press": _diff(fgrid[3], rgrid[3]), "fast": fs, "ref": rs,
                        "centre_shift": float(np.linalg.norm(np.subtract(fs["centre"],
                                                                         rs["centre"]))),
                        "kinetic_rel": abs(fs["kinetic"] - rs["kinetic"]) / max(rs["kinetic"], 1e-30)})
    return {"workload": f"dam_break N={n}, FAST solver (FP32 + FP64 dots, {precond} "
                        f"preconditioner, {arith} gathers) vs the REF step",
            "steps": steps, "rel_tol": rel_tol, "seconds": time.perf_counter() - t0,
            "records": rec}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("which", choices=["pool", "dam_break"])
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--every", type=int, default=None)
    ap.add_argument("--precond", choices=["jacobi", "mg"], default="jacobi",
                    help="dam_break: preconditioner of the FAST solver")
    ap.add_argument("--arith", choices=["ref", "fast"], default="ref",
                    help="dam_break: particle-gather arithmetic of the FAST run")
    a = ap.parse_args(argv)
    gpu.load()
    if a.which == "pool":
        out = pool(a.steps or 200, a.every or 20)
    else:
        out = dam_break(a.steps or 500, a.every or 100, precond=a.precond, arith=a.arith)
    print(json.dumps(out))


if __name__ == "__main__":
    main()

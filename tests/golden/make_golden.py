"""Generate golden vectors by running the reference's own C++.

Builds oracle/_ref/libflipref.so (oracle/Makefile `ref`: the reference
sources compiled where they lie, plus oracle/ref_harness.cpp) and runs its
sorter, mapper, solver, corrector and N=32 driver stages on seeded inputs.
Writes tests/golden/*.npz. Needs the reference tree, so it runs in the build
container only; the committed .npz files travel instead.

Each task runs in its own child process, in a scratch working directory
(the reference appends progress to render/log/console.out and sizes its
solver scratch once per process), with stdout silenced.

    python tests/golden/make_golden.py [task ...]
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libflipref.so")

from flip3d_gb300 import scenes  # noqa: E402

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")

SEED = 7
SUBSET = 4096


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load_ref():
    L = C.CDLL(REF_LIB)
    L.fr_sort.argtypes = [C.c_int, C.c_int, f32p, u8p, u32p, u32p]
    L.fr_mark_water.argtypes = [C.c_int, C.c_int, f32p, u8p, f32p, u8p, f32p]
    L.fr_p2g.argtypes = [C.c_int, C.c_int, f32p, f32p, u8p, f32p, f32p, f32p]
    L.fr_g2p.argtypes = [C.c_int, C.c_int, f32p, u8p, f32p, f32p, f32p, f32p]
    L.fr_solve.argtypes = [C.c_int, C.c_int, C.c_double, u8p, f32p, f32p, f32p]
    L.fr_solve.restype = C.c_int
    L.fr_correct.argtypes = [C.c_int, C.c_int, f32p, f32p, u8p, f32p, C.c_float, C.c_float,
                             C.c_uint64, C.c_int64]
    L.fr_sim_setup.argtypes = [C.c_int, f32p, f32p, u8p, f32p, C.c_float, C.c_uint64,
                               C.c_double]
    L.fr_sim_stage.argtypes = [C.c_int]
    L.fr_sim_get.argtypes = [f32p, f32p, f32p, u8p]
    L.fr_sim_get_grid.argtypes = [f32p, f32p, f32p, u8p, f32p, f32p]
    L.fr_sim_stuck.restype = C.c_int
    L.fr_max_density.restype = C.c_float
    f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
    i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    L.fr_implicit.argtypes = [C.c_int, C.c_int, f32p, u8p, C.c_float, C.c_int, f32p, f64p]
    L.fr_mesh.argtypes = [C.c_int, C.c_int, f32p, u8p, C.c_float, i64p]
    L.fr_sim_mesh.argtypes = [i64p]
    L.fr_mesh_get.argtypes = [f64p, f64p, i32p]
    L.fr_grid_n.restype = C.c_int
    return L


def component_scene(n: int) -> scenes.Scene:
    """A pool+sphere scene with positions and velocities scrambled so that
    clamping, empty cells, crowded cells and close pairs all occur."""
    sc = scenes.pool_sphere(n, seed=SEED)
    rng = np.random.default_rng(SEED)
    fl = sc.type == scenes.FLUID
    pos = sc.pos.copy()
    pos[fl] += rng.normal(0.0, 0.6 / n, size=(fl.sum(), 3)).astype(np.float32)
    # a few particles outside the box (clamping) and a few stacked pairs
    idx = rng.choice(np.nonzero(fl)[0], 40, replace=False)
    pos[idx[:10]] = rng.uniform(-0.2, 1.2, size=(10, 3)).astype(np.float32)
    pos[idx[10:25]] = pos[idx[25:40]] + rng.normal(0, 0.01 / n, size=(15, 3)).astype(np.float32)
    vel = np.where(fl[:, None], rng.normal(0.0, 0.5, size=pos.shape), 0.0).astype(np.float32)
    sc.pos = np.ascontiguousarray(pos)
    sc.vel = np.ascontiguousarray(vel)
    return sc


def task_components(out: str, n: int = 16):
    L = load_ref()
    sc = component_scene(n)
    P = sc.count
    cs = np.zeros(n ** 3 + 1, np.uint32)
    perm = np.zeros(P, np.uint32)
    L.fr_sort(n, P, sc.pos, sc.type, cs, perm)
    rng = np.random.default_rng(SEED + 1)
    dens = np.where(sc.type == scenes.FLUID, rng.uniform(0.0, 0.12, P), 1.0).astype(np.float32)
    A = np.zeros(n ** 3, np.uint8)
    Ls = np.zeros(n ** 3, np.float32)
    L.fr_mark_water(n, P, sc.pos, sc.type, dens, A, Ls)
    fs = (n + 1) * n * n
    u = [np.zeros(fs, np.float32) for _ in range(3)]
    L.fr_p2g(n, P, sc.pos, sc.vel, sc.type, u[0], u[1], u[2])
    grid = [rng.normal(0, 1, fs).astype(np.float32) for _ in range(3)]
    g2p = np.zeros((P, 3), np.float32)
    L.fr_g2p(n, P, sc.pos, sc.type, grid[0], grid[1], grid[2], g2p)
    cpos, cvel = sc.pos.copy(), sc.vel.copy()
    L.fr_correct(n, P, cpos, cvel, sc.type, sc.nrm, np.float32(0.006), np.float32(0.5 / n),
                 SEED, 3)
    np.savez_compressed(out, n=n, pos=sc.pos, vel=sc.vel, type=sc.type, nrm=sc.nrm,
                        cell_start=cs, perm=perm, dens=dens, A=A, L=Ls, u0=u[0], u1=u[1],
                        u2=u[2], grid0=grid[0], grid1=grid[1], grid2=grid[2], g2p=g2p,
                        corr_pos=cpos, corr_vel=cvel, corr_seed=SEED, corr_step=3)


def task_solver(out: str, n: int = 16):
    L = load_ref()
    from oracle import pyoracle as orc  # the oracle only prepares a realistic input
    sc = scenes.pool_sphere(n, seed=SEED)
    cs, perm = orc.sort(n, sc.pos)
    md = orc.max_density(n)
    dens = orc.density(n, sc.pos, sc.type, cs, perm, md)
    A = orc.mark_water(n, sc.type, dens, cs, perm)
    Ls = orc.levelset(n, sc.type, dens, cs, perm)
    rng = np.random.default_rng(SEED + 2)
    b = np.where(A == 1, rng.normal(0, 3.0, n ** 3), rng.normal(0, 1, n ** 3)).astype(np.float32)
    x0 = np.where(A == 1, rng.normal(0, 0.02, n ** 3), 0).astype(np.float32)
    res = {}
    for tag, rel in (("abs", 0.0), ("rel6", 1e-6)):
        x = x0.copy()
        bb = b.copy()
        k = L.fr_solve(n, 1, rel, A, Ls, x, bb)
        res[f"x_{tag}"] = x
        res[f"b_{tag}"] = bb
        res[f"k_{tag}"] = k
    np.savez_compressed(out, n=n, A=A, L=Ls, x0=x0, b=b, **res)


def task_driver(out: str, steps: int = 10, rel_tol: float = 1e-6):
    L = load_ref()
    n = L.fr_grid_n()
    sc = scenes.pool_sphere(n, seed=0)
    md = L.fr_max_density()
    L.fr_sim_setup(sc.count, sc.pos, sc.vel, sc.type, sc.nrm, md, SEED, rel_tol)
    P = sc.count
    fs = (n + 1) * n * n
    rng = np.random.default_rng(SEED + 3)
    sub = np.sort(rng.choice(P, min(SUBSET, P), replace=False))
    rec = {"n": n, "max_dens": np.float32(md), "seed": SEED, "rel_tol": rel_tol,
           "steps": steps, "subset": sub, "scene_pos_sha": digest(sc.pos)}

    def snap(tag):
        pos = np.zeros((P, 3), np.float32)
        vel = np.zeros((P, 3), np.float32)
        dens = np.zeros(P, np.float32)
        typ = np.zeros(P, np.uint8)
        L.fr_sim_get(pos, vel, dens, typ)
        u = [np.zeros(fs, np.float32) for _ in range(3)]
        A = np.zeros(n ** 3, np.uint8)
        Ls = np.zeros(n ** 3, np.float32)
        pr = np.zeros(n ** 3, np.float32)
        L.fr_sim_get_grid(u[0], u[1], u[2], A, Ls, pr)
        fluid = typ == 1
        for name, arr in (("pos", pos), ("vel_fluid", np.where(fluid[:, None], vel, 0)),
                          ("dens", dens), ("u0", u[0]), ("u1", u[1]), ("u2", u[2]), ("A", A),
                          ("L", Ls), ("press", pr)):
            arr = np.ascontiguousarray(arr)
            rec[f"{tag}_{name}_sha"] = digest(arr)
            if arr.shape[0] == P:
                rec[f"{tag}_{name}_sub"] = arr[sub]
            else:
                rec[f"{tag}_{name}_sub"] = arr[:: max(1, arr.shape[0] // SUBSET)]
        rec[f"{tag}_stuck"] = L.fr_sim_stuck()

    for st in range(5):
        L.fr_sim_stage(st)
        snap(f"s1_stage{st}")
    for k in range(2, steps + 1):
        for st in range(5):
            L.fr_sim_stage(st)
        if k in (2, 5, steps):
            snap(f"step{k}")
    np.savez_compressed(out, **rec)


def load_ref64(n: int):
    """The FP64 oracle: the reference built with FLOAT = double and its
    driver's N = n (oracle/build_ref64.sh)."""
    path = os.path.join(ROOT, "oracle", "_ref", f"libflipref64_n{n}.so")
    subprocess.check_call(["sh", os.path.join(ROOT, "oracle", "build_ref64.sh"), str(n)],
                          stdout=subprocess.DEVNULL)
    L = C.CDLL(path)
    f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    L.fr_sim_setup.argtypes = [C.c_int, f32p, f32p, u8p, f32p, C.c_float, C.c_uint64,
                               C.c_double]
    L.fr_sim_stage.argtypes = [C.c_int]
    L.fr_sim_get.argtypes = [f32p, f32p, f32p, u8p]
    L.fr_sim_get_d.argtypes = [f64p, f64p, f64p]
    L.fr_sim_get_grid_d.argtypes = [f64p, f64p, f64p, f64p, f64p]
    L.fr_sim_get_grid.argtypes = [f32p, f32p, f32p, u8p, f32p, f32p]
    L.fr_max_density_d.restype = C.c_double
    L.fr_sim_set_max_density_d.argtypes = [C.c_double]
    L.fr_grid_n.restype = C.c_int
    return L


# FP64 runs: (scene, snapshot steps). The N=32 pool + sphere for 200 steps
# and the N=128 dam break for its first 50 steps (an FP64 step of the
# reference at N=128 takes about a minute on eight cores).
FP64_RUNS = {32: ("pool_sphere", (1, 10, 50, 200)), 128: ("dam_break", (1, 5, 10, 25, 50))}


def task_fp64(out: str, n: int):
    """The reference's own step in FP64 from a seeded scene: particle
    subsets, pressure and face velocities on the i = n/4 plane, and
    full-set aggregates at the snapshot steps."""
    L = load_ref64(n)
    assert L.fr_grid_n() == n
    scene, snaps = FP64_RUNS[n]
    sc = getattr(scenes, scene)(n, seed=0)
    md = L.fr_max_density_d()
    L.fr_sim_setup(sc.count, sc.pos, sc.vel, sc.type, sc.nrm, np.float32(md), SEED, 1e-6)
    L.fr_sim_set_max_density_d(md)
    P = sc.count
    fs = (n + 1) * n * n
    rng = np.random.default_rng(SEED + 5)
    sub = np.sort(rng.choice(P, min(SUBSET, P), replace=False))
    fluid = sc.type == 1
    # the i = n/4 plane: through the liquid of both scenes (the dam break's
    # column ends at x = 0.4)
    plane_i = n // 4
    rec = {"n": n, "scene": scene, "seed": SEED, "rel_tol": 1e-6, "max_dens": md,
           "snaps": np.array(snaps), "subset": sub, "scene_pos_sha": digest(sc.pos),
           "count": P, "plane": plane_i}

    def plane(a, shape):
        return np.ascontiguousarray(a.reshape(shape)[plane_i])

    def snap(k):
        pos = np.zeros((P, 3), np.float64)
        vel = np.zeros((P, 3), np.float64)
        dens = np.zeros(P, np.float64)
        L.fr_sim_get_d(pos, vel, dens)
        u = [np.zeros(fs, np.float64) for _ in range(3)]
        Ls = np.zeros(n ** 3, np.float64)
        pr = np.zeros(n ** 3, np.float64)
        L.fr_sim_get_grid_d(u[0], u[1], u[2], Ls, pr)
        A = np.zeros(n ** 3, np.uint8)
        L.fr_sim_get_grid(np.zeros(fs, np.float32), np.zeros(fs, np.float32),
                          np.zeros(fs, np.float32), A, np.zeros(n ** 3, np.float32),
                          np.zeros(n ** 3, np.float32))
        t = f"step{k}"
        rec[f"{t}_pos"] = pos[sub]
        rec[f"{t}_vel"] = np.where(fluid[sub, None], vel[sub], 0.0)
        rec[f"{t}_dens"] = dens[sub]
        rec[f"{t}_press"] = plane(pr, (n, n, n))
        rec[f"{t}_A"] = plane(A, (n, n, n))
        rec[f"{t}_u0"] = plane(u[0], (n + 1, n, n))
        rec[f"{t}_u1"] = plane(u[1], (n, n + 1, n))
        rec[f"{t}_u2"] = plane(u[2], (n, n, n + 1))
        fp, fv = pos[fluid], vel[fluid]
        rec[f"{t}_com"] = fp.mean(axis=0)
        rec[f"{t}_ke"] = 0.5 * float((fv * fv).sum()) / fp.shape[0]
        rec[f"{t}_pmax"] = float(np.abs(pr).max())

    for k in range(1, max(snaps) + 1):
        for st in range(5):
            L.fr_sim_stage(st)
        if k in snaps:
            snap(k)
    np.savez_compressed(out, **rec)


def _mesh_arrays(L, counts):
    nv, nf = int(counts[0]), int(counts[1])
    v = np.zeros(3 * nv, np.float64)
    nr = np.zeros(3 * nv, np.float64)
    f = np.zeros(3 * nf, np.int32)
    L.fr_mesh_get(v, nr, f)
    return v, nr, f


def task_mesh(out: str, n: int):
    """generateMesh (mg = n+1) and implicit_func on the scrambled scene."""
    L = load_ref()
    sc = component_scene(n)
    P = sc.count
    rng = np.random.default_rng(SEED + 4)
    pts = rng.uniform(-0.1, 1.1, size=(3000, 3)).astype(np.float32)
    pts[:1000] = sc.pos[rng.choice(P, 1000, replace=False)] + \
        rng.normal(0, 0.3 / n, size=(1000, 3)).astype(np.float32)
    phi = np.zeros(pts.shape[0], np.float64)
    L.fr_implicit(n, P, sc.pos, sc.type, np.float32(0.5), pts.shape[0], pts, phi)
    counts = np.zeros(2, np.int64)
    L.fr_mesh(n, P, sc.pos, sc.type, np.float32(0.5), counts)
    v, nr, f = _mesh_arrays(L, counts)
    np.savez_compressed(out, n=n, pos=sc.pos, type=sc.type, pts=pts, phi=phi, vertices=v,
                        normals=nr, faces=f)


def task_export(out: str, n: int = 16, frame: int = 7):
    """exporter::write3D on the mesh of the mesh_n16 task's scene: digests and
    sizes of the OBJ and Sunflow scene files it writes."""
    L = load_ref()
    L.fr_export.argtypes = [C.c_int, C.c_float]
    sc = component_scene(n)
    counts = np.zeros(2, np.int64)
    L.fr_mesh(n, sc.count, sc.pos, sc.type, np.float32(0.5), counts)
    v, nr, f = _mesh_arrays(L, counts)
    wt = np.float32(1.0 / n)
    L.fr_export(frame, wt)
    rec = {"n": n, "frame": frame, "wall_thick": wt, "counts": counts}
    for tag, path in (("obj", f"render/obj/{frame}_scene.obj"),
                      ("sunflow", f"render/sunflow/{frame}_scene.sc")):
        raw = open(path, "rb").read()
        rec[f"{tag}_sha256"] = hashlib.sha256(raw).hexdigest()
        rec[f"{tag}_bytes"] = len(raw)
        rec[f"{tag}_head"] = np.frombuffer(raw[:512], np.uint8)
    rec["mesh_sha256"] = hashlib.sha256(v.tobytes() + nr.tobytes() + f.tobytes()).hexdigest()
    np.savez_compressed(out, **rec)


def task_preview(out: str):
    """write_frame's BMP (1024 x 700, step 0) for two N=32 scenes set up in the
    driver: digests and sizes."""
    L = load_ref()
    n = L.fr_grid_n()
    md = L.fr_max_density()
    rec = {"n": n}
    for tag, sc in (("pool_sphere", scenes.pool_sphere(n, seed=0)),
                    ("random_s5", scenes.random_scene(n, 5))):
        L.fr_sim_setup(sc.count, sc.pos, sc.vel, sc.type, sc.nrm, md, SEED, 1e-6)
        L.fr_write_frame()
        raw = open(os.path.join("render", "preview", "frame_0.bmp"), "rb").read()
        rec[f"{tag}_sha256"] = hashlib.sha256(raw).hexdigest()
        rec[f"{tag}_bytes"] = len(raw)
        rec[f"{tag}_covered"] = int((np.frombuffer(raw[54:], np.uint8) > 0).sum())
    np.savez_compressed(out, **rec)


def task_mesh_driver(out: str, steps: int = 3):
    """The mesh write_mesh makes after `steps` driver steps at N=32: digests
    and subsets (the oracle rebuilds the state by running its own steps)."""
    L = load_ref()
    n = L.fr_grid_n()
    sc = scenes.pool_sphere(n, seed=0)
    md = L.fr_max_density()
    L.fr_sim_setup(sc.count, sc.pos, sc.vel, sc.type, sc.nrm, md, SEED, 1e-6)
    for _ in range(steps):
        for st in range(5):
            L.fr_sim_stage(st)
    counts = np.zeros(2, np.int64)
    L.fr_sim_mesh(counts)
    v, nr, f = _mesh_arrays(L, counts)
    rng = np.random.default_rng(SEED + 5)
    sv = np.sort(rng.choice(v.shape[0], min(3000, v.shape[0]), replace=False))
    sf = np.sort(rng.choice(f.shape[0], min(3000, f.shape[0]), replace=False))
    np.savez_compressed(out, n=n, steps=steps, seed=SEED, rel_tol=1e-6, counts=counts,
                        vertices_sha=digest(v), normals_sha=digest(nr), faces_sha=digest(f),
                        vsub=sv, vertices_sub=v[sv], normals_sub=nr[sv], fsub=sf,
                        faces_sub=f[sf])


CKPT_RECORD = np.dtype([("p", "<f4", 3), ("u", "<f4", 3), ("n", "<f4", 3), ("type", "i1"),
                        ("visible", "i1"), ("remove", "i1"), ("thin", "i1"),
                        ("tmp", "<f4", 6), ("m", "<f4"), ("dens", "<f4")])


def checkpoint_canonical(raw: bytes, n: int):
    """Parse a reference checkpoint (src/flip3D.cpp:453-516) and zero the
    bytes the reference leaves undefined: each record's tmp[2][3] (scratch,
    partly never initialised) and remove (not set by pushParticle), and the
    wall normals of cells that are neither wall nor perimeter cells
    (allocated without initialisation when no particle visits them)."""
    assert CKPT_RECORD.itemsize == 72
    count = int(np.frombuffer(raw, "<i4", 1, 0)[0])
    parts = np.frombuffer(raw, CKPT_RECORD, count, 24).copy()
    off = 24 + 72 * count
    press = np.frombuffer(raw, "<f4", n ** 3, off).copy()
    wn = np.frombuffer(raw, "<f4", 4 * n ** 3, off + 4 * n ** 3).reshape(n ** 3, 4).copy()
    assert len(raw) == off + 20 * n ** 3
    wall = np.zeros(n ** 3, bool)
    w = parts[parts["type"] == 2]["p"]
    c = np.clip(w * np.float32(n), 0, n - 1).astype(np.int64)
    wall[(c[:, 0] * n + c[:, 1]) * n + c[:, 2]] = True
    other = ~wall & (wn[:, 3] != 1.0)
    wn[other, :3] = 0.0
    parts["tmp"] = 0.0
    parts["remove"] = 0
    canonical = raw[:24] + parts.tobytes() + press.tobytes() + wn.tobytes()
    return parts, press, wn, canonical


def task_checkpoint(out: str):
    """The reference's own init + saveState at N=32 (its damBreakTest scene):
    the parsed content and the digest of the canonical bytes."""
    L = load_ref()
    L.fr_init_and_save.restype = C.c_int
    L.fr_init_and_save.argtypes = [C.c_uint64]
    count = L.fr_init_and_save(SEED)
    n = L.fr_grid_n()
    with open(os.path.join("render", "save", "0_scene.dat"), "rb") as f:
        raw = f.read()
    parts, press, wn, canonical = checkpoint_canonical(raw, n)
    assert parts.shape[0] == count
    hdr = np.frombuffer(raw, "<f4", 6, 0)
    np.savez_compressed(
        out, n=n, count=count, max_dens=hdr[1], pour_time=np.frombuffer(raw, "<i4", 1, 8)[0],
        pour_pos=hdr[3:5], pour_rad=hdr[5], pos=parts["p"], vel=parts["u"], nrm=parts["n"],
        type=parts["type"].astype(np.uint8), visible=parts["visible"].astype(np.uint8),
        thin=parts["thin"].astype(np.uint8), m=parts["m"], dens=parts["dens"], press=press,
        wall_normal=wn, canonical_sha256=hashlib.sha256(canonical).hexdigest(),
        file_bytes=len(raw))


TASKS = {
    "components_n16": lambda out: task_components(out, 16),
    "components_n13": lambda out: task_components(out, 13),
    "solver_n16": lambda out: task_solver(out, 16),
    "solver_n13": lambda out: task_solver(out, 13),
    "driver_n32": lambda out: task_driver(out, 10, 1e-6),
    "driver_n32_abs": lambda out: task_driver(out, 5, 0.0),
    "mesh_n16": lambda out: task_mesh(out, 16),
    "mesh_n13": lambda out: task_mesh(out, 13),
    "mesh_driver_n32": lambda out: task_mesh_driver(out, 3),
    "checkpoint_n32": task_checkpoint,
    "export_n16": task_export,
    "preview_n32": task_preview,
    "fp64_n32": lambda out: task_fp64(out, 32),
    "fp64_n128": lambda out: task_fp64(out, 128),
}


def run_child(task: str, out: str):
    os.chdir(tempfile.mkdtemp(prefix="flipref_"))
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    os.environ["OMP_NUM_THREADS"] = "1"
    TASKS[task](out)


def main(argv):
    if len(argv) >= 3 and argv[1] == "--child":
        run_child(argv[2], argv[3])
        return
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    tasks = argv[1:] or list(TASKS)
    env = dict(os.environ, OMP_NUM_THREADS="1")
    for t in tasks:
        out = os.path.join(HERE, f"{t}.npz")
        subprocess.check_call([sys.executable, os.path.abspath(__file__), "--child", t, out],
                              env=env)
        print(f"wrote {out} ({os.path.getsize(out) // 1024} KiB)")


if __name__ == "__main__":
    main(sys.argv)

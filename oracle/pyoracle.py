"""ctypes access to the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the flip3d_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")

PRECOND_NONE, PRECOND_REF, PRECOND_IC = 0, 1, 2


class OrcParams(C.Structure):
    _fields_ = [("n", C.c_int), ("density", C.c_float), ("alpha", C.c_double),
                ("dt", C.c_double), ("gravity", C.c_double), ("subcell", C.c_int),
                ("precond", C.c_int), ("mic_tau", C.c_double), ("eps_abs", C.c_double),
                ("rel_tol", C.c_double), ("max_iters", C.c_int), ("seed", C.c_uint64)]


def params(n, precond=PRECOND_REF, rel_tol=0.0, eps_abs=-1.0, mic_tau=0.0, dt=0.006,
           seed=0, max_iters=0, subcell=1):
    return OrcParams(n, 0.5, 0.95, dt, 9.8, subcell, precond, mic_tau, eps_abs, rel_tol,
                     max_iters, seed)


def build():
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_sort.argtypes = [C.c_int, C.c_int, f32p, u32p, u32p]
        L.orc_density.argtypes = [C.c_int, C.c_int, f32p, u8p, u32p, u32p, C.c_float,
                                  C.c_float, f32p]
        L.orc_levelset.argtypes = [C.c_int, u8p, f32p, u32p, u32p, C.c_float, f32p]
        L.orc_mark_water.argtypes = [C.c_int, u8p, f32p, u32p, u32p, C.c_float, u8p]
        L.orc_p2g.argtypes = [C.c_int, C.c_int, f32p, f32p, u8p, u32p, u32p, f32p, f32p, f32p]
        L.orc_g2p.argtypes = [C.c_int, C.c_int, f32p, u8p, f32p, f32p, f32p, f32p, C.c_int]
        L.orc_enforce_boundary.argtypes = [C.c_int, u8p, f32p, f32p, f32p]
        L.orc_divergence.argtypes = [C.c_int, u8p, f32p, f32p, f32p, f32p]
        L.orc_subtract_gradient.argtypes = [C.c_int, C.c_int, f32p, f32p, f32p, f32p, f32p]
        L.orc_extrapolate.argtypes = [C.c_int, u8p, f32p, f32p, f32p]
        L.orc_solve.argtypes = [C.POINTER(OrcParams), u8p, f32p, f32p, f32p,
                                C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_solve.restype = C.c_int
        L.orc_precond_apply.argtypes = [C.POINTER(OrcParams), u8p, f32p, f32p, f32p]
        L.orc_matvec.argtypes = [C.c_int, C.c_int, u8p, f32p, f32p, f32p]
        L.orc_correct.argtypes = [C.c_int, C.c_int, f32p, f32p, u8p, f32p, u32p, u32p,
                                  C.c_float, C.c_float, C.c_uint64, C.c_int64]
        L.orc_resample.argtypes = [C.c_int, f32p, f32p, u8p, u32p, u32p, f32p, f32p, C.c_float]
        L.orc_sim_create.argtypes = [C.POINTER(OrcParams), C.c_int, f32p, f32p, u8p, f32p,
                                     C.c_float]
        L.orc_sim_create.restype = C.c_void_p
        L.orc_sim_destroy.argtypes = [C.c_void_p]
        L.orc_sim_step.argtypes = [C.c_void_p]
        L.orc_sim_step.restype = C.c_int
        L.orc_sim_stage.argtypes = [C.c_void_p, C.c_int]
        L.orc_sim_get.argtypes = [C.c_void_p, f32p, f32p, f32p, u8p]
        L.orc_sim_get_grid.argtypes = [C.c_void_p, f32p, f32p, f32p, u8p, f32p, f32p]
        L.orc_sim_put.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_sim_put_grid.argtypes = [C.c_void_p] + [C.c_void_p] * 6
        L.orc_sim_last_stuck.argtypes = [C.c_void_p]
        L.orc_sim_last_stuck.restype = C.c_int
        L.orc_sim_last_r2.argtypes = [C.c_void_p]
        L.orc_sim_last_r2.restype = C.c_double
        L.orc_sim_set_step.argtypes = [C.c_void_p, C.c_int64]
        L.orc_sim_set_threads.argtypes = [C.c_int]
        L.orc_implicit.argtypes = [C.c_int, f32p, u8p, u32p, u32p, C.c_float, C.c_int, f32p,
                                   f64p]
        L.orc_mesh.argtypes = [C.c_int, f32p, u8p, u32p, u32p, C.c_float]
        L.orc_mesh.restype = C.c_void_p
        L.orc_sim_mesh.argtypes = [C.c_void_p]
        L.orc_sim_mesh.restype = C.c_void_p
        L.orc_mesh_counts.argtypes = [C.c_void_p] + [C.POINTER(C.c_int64)] * 3
        L.orc_mesh_get.argtypes = [C.c_void_p, f64p, f64p, i32p, f32p]
        L.orc_mesh_free.argtypes = [C.c_void_p]
        L.orc_max_density.argtypes = [C.c_int, C.c_float]
        L.orc_max_density.restype = C.c_float
        _lib = L
    return _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def sort(n, pos):
    pos = _c(pos, np.float32)
    cs = np.zeros(n ** 3 + 1, np.uint32)
    perm = np.zeros(pos.shape[0], np.uint32)
    lib().orc_sort(n, pos.shape[0], pos, cs, perm)
    return cs, perm


def density(n, pos, typ, cs, perm, max_dens, density_param=0.5):
    out = np.zeros(pos.shape[0], np.float32)
    kh = np.float32(4.0 * density_param / n)
    lib().orc_density(n, pos.shape[0], _c(pos, np.float32), _c(typ, np.uint8), cs, perm,
                      kh, np.float32(max_dens), out)
    return out


def levelset(n, typ, dens, cs, perm):
    L = np.zeros(n ** 3, np.float32)
    lib().orc_levelset(n, _c(typ, np.uint8), _c(dens, np.float32), cs, perm, 0.5, L)
    return L


def mark_water(n, typ, dens, cs, perm):
    A = np.zeros(n ** 3, np.uint8)
    lib().orc_mark_water(n, _c(typ, np.uint8), _c(dens, np.float32), cs, perm, 0.5, A)
    return A


def face_shapes(n):
    return (n + 1) * n * n


def p2g(n, pos, vel, typ, cs, perm):
    u = [np.zeros(face_shapes(n), np.float32) for _ in range(3)]
    lib().orc_p2g(n, pos.shape[0], _c(pos, np.float32), _c(vel, np.float32),
                  _c(typ, np.uint8), cs, perm, u[0], u[1], u[2])
    return u


def g2p(n, pos, typ, u, fluid_only=False):
    vel = np.zeros((pos.shape[0], 3), np.float32)
    lib().orc_g2p(n, pos.shape[0], _c(pos, np.float32), _c(typ, np.uint8),
                  _c(u[0], np.float32), _c(u[1], np.float32), _c(u[2], np.float32),
                  vel, int(fluid_only))
    return vel


def matvec(n, A, L, x, subcell=1):
    out = np.zeros(n ** 3, np.float32)
    lib().orc_matvec(n, subcell, _c(A, np.uint8), _c(L, np.float32), _c(x, np.float32), out)
    return out


def solve(prm, A, L, x, b):
    x = _c(x, np.float32).copy()
    b = _c(b, np.float32).copy()
    r2 = C.c_double(0)
    b2 = C.c_double(0)
    it = lib().orc_solve(C.byref(prm), _c(A, np.uint8), _c(L, np.float32), x, b,
                         C.byref(r2), C.byref(b2))
    return x, b, it, r2.value, b2.value


def precond_apply(prm, A, L, r):
    z = np.zeros_like(_c(r, np.float32))
    lib().orc_precond_apply(C.byref(prm), _c(A, np.uint8), _c(L, np.float32),
                            _c(r, np.float32), z)
    return z


def correct(n, pos, vel, typ, nrm, cs, perm, dt, re, seed, step):
    pos = _c(pos, np.float32).copy()
    vel = _c(vel, np.float32).copy()
    lib().orc_correct(n, pos.shape[0], pos, vel, _c(typ, np.uint8), _c(nrm, np.float32),
                      cs, perm, np.float32(dt), np.float32(re), seed, step)
    return pos, vel


def resample(n, pos, vel, typ, cs, perm, p, u, re):
    """corrector::resample at one point; u is the fallback velocity."""
    out = _c(u, np.float32).copy()
    lib().orc_resample(n, _c(pos, np.float32), _c(vel, np.float32), _c(typ, np.uint8),
                       _c(cs, np.uint32), _c(perm, np.uint32), _c(p, np.float32), out,
                       np.float32(re))
    return out


def implicit(n, pos, typ, cs, perm, pts, density=0.5):
    """implicit::implicit_func at each point of pts [m,3]."""
    pts = _c(pts, np.float32)
    out = np.zeros(pts.shape[0], np.float64)
    lib().orc_implicit(n, _c(pos, np.float32), _c(typ, np.uint8), _c(cs, np.uint32),
                       _c(perm, np.uint32), np.float32(density), pts.shape[0], pts, out)
    return out


def _take_mesh(h, n):
    L = lib()
    nv, nf, nt = C.c_int64(), C.c_int64(), C.c_int64()
    L.orc_mesh_counts(h, C.byref(nv), C.byref(nf), C.byref(nt))
    out = {"vertices": np.zeros(3 * nv.value, np.float64),
           "normals": np.zeros(3 * nv.value, np.float64),
           "faces": np.zeros(3 * nf.value, np.int32),
           "phi": np.zeros((n + 1) ** 3, np.float32), "triangles": nt.value}
    L.orc_mesh_get(h, out["vertices"], out["normals"], out["faces"], out["phi"])
    L.orc_mesh_free(h)
    return out


def mesh(n, pos, typ, cs, perm, density=0.5):
    """mesher::generateMesh with mg = n+1: dict of vertices, normals (flat
    float64), faces (flat int32), phi ((n+1)^3, x fastest), triangles."""
    h = lib().orc_mesh(n, _c(pos, np.float32), _c(typ, np.uint8), _c(cs, np.uint32),
                       _c(perm, np.uint32), np.float32(density))
    return _take_mesh(h, n)


def max_density(n, density_param=0.5):
    return float(lib().orc_max_density(n, np.float32(density_param)))


class Sim:
    """Stateful oracle simulation (one simulateStep per ``step()``)."""

    def __init__(self, scene, prm, max_dens=None):
        self.n = scene.n
        md = max_density(scene.n) if max_dens is None else max_dens
        self.np = scene.count
        self._h = lib().orc_sim_create(C.byref(prm), self.np, _c(scene.pos, np.float32),
                                       _c(scene.vel, np.float32), _c(scene.type, np.uint8),
                                       _c(scene.nrm, np.float32), np.float32(md))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_sim_destroy(self._h)
            self._h = None

    def step(self):
        return lib().orc_sim_step(self._h)

    def stage(self, s):
        lib().orc_sim_stage(self._h, s)

    def set_step(self, s):
        lib().orc_sim_set_step(self._h, s)

    def get(self):
        pos = np.zeros((self.np, 3), np.float32)
        vel = np.zeros((self.np, 3), np.float32)
        dens = np.zeros(self.np, np.float32)
        typ = np.zeros(self.np, np.uint8)
        lib().orc_sim_get(self._h, pos, vel, dens, typ)
        return pos, vel, dens, typ

    def grid(self):
        n = self.n
        u = [np.zeros(face_shapes(n), np.float32) for _ in range(3)]
        A = np.zeros(n ** 3, np.uint8)
        L = np.zeros(n ** 3, np.float32)
        p = np.zeros(n ** 3, np.float32)
        lib().orc_sim_get_grid(self._h, u[0], u[1], u[2], A, L, p)
        return u, A, L, p

    def put(self, pos=None, vel=None, dens=None):
        keep = [None if a is None else _c(a, np.float32) for a in (pos, vel, dens)]
        lib().orc_sim_put(self._h, *[None if a is None else a.ctypes.data for a in keep])

    def put_grid(self, u=None, A=None, L=None, press=None):
        u = [None] * 3 if u is None else list(u)
        keep = [None if a is None else _c(a, np.float32) for a in u]
        keep.append(None if A is None else _c(A, np.uint8))
        keep += [None if a is None else _c(a, np.float32) for a in (L, press)]
        lib().orc_sim_put_grid(self._h, *[None if a is None else a.ctypes.data for a in keep])

    def mesh(self):
        return _take_mesh(lib().orc_sim_mesh(self._h), self.n)

    @property
    def stuck(self):
        return lib().orc_sim_last_stuck(self._h)


def set_threads(n):
    lib().orc_sim_set_threads(n)


def fast_diag(n, A, L, subcell=1):
    """Diagonal of the FAST-mode pressure operator: A_diag of
    src/solver.cpp:103-117 in float with the reference's double promotions,
    neighbours in the order i-1, i+1, j-1, j+1, k-1, k+1 (a wall or the
    domain's edge subtracts 1, an air cell L_q / min(1e-6, L_c))."""
    A3 = np.asarray(A, np.uint8).reshape(n, n, n)
    L3 = np.asarray(L, np.float32).reshape(n, n, n).astype(np.float64)
    Lc = np.fmin(1.0e-6, L3)
    diag = np.full((n, n, n), 6.0, np.float32)
    Ap = np.pad(A3, 1, constant_values=2)  # outside the grid counts as wall
    Lp = np.pad(L3, 1)
    for axis in range(3):
        for step in (-1, 1):
            sl = [slice(1, n + 1)] * 3
            sl[axis] = slice(1 + step, n + 1 + step)
            an, ln = Ap[tuple(sl)], Lp[tuple(sl)]
            wall = an == 2
            air = (an == 0) & bool(subcell)
            d = diag.astype(np.float64)
            diag = np.where(wall, (d - 1.0).astype(np.float32),
                            np.where(air, (d - ln / Lc).astype(np.float32), diag))
    return diag.reshape(-1)


def fast_residual_fp64(n, A, L, b, x, subcell=1):
    """b - M x in FP64 for the FAST-mode operator M = (diag*x - sum of the
    fluid neighbours' x) * inv_h2 (its FP32 coefficients taken exactly), on
    the fluid cells; zero elsewhere. x may be float64 (a refined iterate)."""
    A3 = np.asarray(A, np.uint8).reshape(n, n, n)
    fl = A3 == 1
    x3 = np.where(fl, np.asarray(x, np.float64).reshape(n, n, n), 0.0)
    diag = fast_diag(n, A, L, subcell).reshape(n, n, n).astype(np.float64)
    h2f = np.float32(1.0 / (float(n) * n))
    inv_h2_f = float(np.float32(1.0 / float(h2f)))
    xp = np.pad(x3, 1)
    nb = np.zeros_like(x3)
    for axis in range(3):
        for step in (-1, 1):
            sl = [slice(1, n + 1)] * 3
            sl[axis] = slice(1 + step, n + 1 + step)
            nb += xp[tuple(sl)]
    ax = (diag * x3 - nb) * inv_h2_f
    r = np.where(fl, np.asarray(b, np.float32).reshape(n, n, n).astype(np.float64) - ax, 0.0)
    return r.reshape(-1)

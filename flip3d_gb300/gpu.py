"""Python access to libflipgpu.so through its C ABI (include/flipgpu.h).

There is no CPU path: constructing a Simulation without the CUDA library or
without a GPU raises.
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB

OK = 0
ERRORS = {-1: "EINVAL", -2: "ECUDA", -3: "ENOMEM", -4: "ENOCONV", -5: "ENAN", -6: "ETIMEOUT",
          -7: "ETOOBIG"}
PRECOND_NONE, PRECOND_REF, PRECOND_IC, PRECOND_JACOBI, PRECOND_MG = 0, 1, 2, 3, 4
SOLVE_REF, SOLVE_FAST = 0, 1
ARITH_REF, ARITH_FAST = 0, 1

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")


class Params(C.Structure):
    _fields_ = [("n", C.c_int), ("max_particles", C.c_int), ("density", C.c_float),
                ("alpha", C.c_double), ("dt", C.c_double), ("gravity", C.c_double),
                ("subcell", C.c_int), ("seed", C.c_uint64), ("solve_mode", C.c_int),
                ("precond", C.c_int), ("mic_tau", C.c_double), ("rel_tol", C.c_double),
                ("eps_abs", C.c_double), ("max_iters", C.c_int), ("refine_steps", C.c_int),
                ("arith", C.c_int), ("mg_sweeps", C.c_int)]


class SceneObject(C.Structure):
    _fields_ = [("shape", C.c_int), ("lo", C.c_float * 3), ("hi", C.c_float * 3),
                ("c", C.c_float * 3), ("r", C.c_float), ("vel", C.c_float * 3)]


class Checkpoint(C.Structure):
    _fields_ = [("n", C.c_int), ("count", C.c_int), ("max_dens", C.c_float),
                ("pour_time", C.c_int), ("pour_pos", C.c_float * 2), ("pour_rad", C.c_float),
                ("pos", C.c_void_p), ("vel", C.c_void_p), ("nrm", C.c_void_p),
                ("type", C.c_void_p), ("visible", C.c_void_p), ("dens", C.c_void_p),
                ("press", C.c_void_p), ("wall_normal", C.c_void_p)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("status", C.c_int), ("r2", C.c_double),
                ("b2", C.c_double), ("ms", C.c_double), ("warm", C.c_int),
                ("r2_prev", C.c_double), ("r2_guess", C.c_double), ("gamma", C.c_double),
                ("warm_ms", C.c_double), ("r2_true", C.c_double), ("refine_passes", C.c_int)]


class FlipGpuError(RuntimeError):
    pass


_lib = None

# every exported entry point and its argument types
SIGNATURES = {
    "flipgpu_default_params": (None, [C.POINTER(Params), C.c_int, C.c_int]),
    "flipgpu_create": (C.c_int, [C.POINTER(Params), C.POINTER(C.c_void_p)]),
    "flipgpu_destroy": (C.c_int, [C.c_void_p]),
    "flipgpu_last_error": (C.c_char_p, [C.c_void_p]),
    "flipgpu_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "flipgpu_sync": (C.c_int, [C.c_void_p]),
    "flipgpu_set_step": (C.c_int, [C.c_void_p, C.c_int64]),
    "flipgpu_seed_scene": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_uint64, C.c_double,
                                     C.c_double]),
    "flipgpu_particle_count": (C.c_int, [C.c_void_p]),
    "flipgpu_write_obj": (C.c_int, [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                    C.c_int64, C.c_float]),
    "flipgpu_write_sunflow": (C.c_int, [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int64,
                                        C.c_void_p, C.c_int64, C.c_float]),
    "flipgpu_export_mesh": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.c_float, C.c_int,
                                      C.c_char_p]),
    "flipgpu_export_wait": (C.c_int, [C.c_void_p]),
    "flipgpu_preview": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "flipgpu_set_autotune": (C.c_int, [C.c_int]),
    "flipgpu_autotune_report": (C.c_int, [C.c_char_p, C.c_int]),
    "flipgpu_write_bmp": (C.c_int, [C.c_char_p, C.c_void_p, C.c_int, C.c_int]),
    "flipgpu_checkpoint_write": (C.c_int, [C.c_char_p, C.c_void_p]),
    "flipgpu_checkpoint_count": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_int)]),
    "flipgpu_checkpoint_read": (C.c_int, [C.c_char_p, C.c_void_p]),
    "flipgpu_save_state": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.c_void_p, C.c_float]),
    "flipgpu_load_state": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_int), C.c_void_p,
                                     C.POINTER(C.c_float)]),
    "flipgpu_set_particles": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_int]),
    "flipgpu_get_particles": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_int]),
    "flipgpu_count": (C.c_int, [C.c_void_p]),
    "flipgpu_set_grid": (C.c_int, [C.c_void_p] + [C.c_void_p] * 7 + [C.c_int]),
    "flipgpu_get_grid": (C.c_int, [C.c_void_p] + [C.c_void_p] * 7 + [C.c_int]),
    "flipgpu_get_cells": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "flipgpu_set_max_density": (C.c_int, [C.c_void_p, C.c_float]),
    "flipgpu_calibrate_max_density": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "flipgpu_sort": (C.c_int, [C.c_void_p]),
    "flipgpu_compute_density": (C.c_int, [C.c_void_p]),
    "flipgpu_mark_water": (C.c_int, [C.c_void_p]),
    "flipgpu_add_force": (C.c_int, [C.c_void_p]),
    "flipgpu_p2g": (C.c_int, [C.c_void_p]),
    "flipgpu_g2p": (C.c_int, [C.c_void_p]),
    "flipgpu_solve": (C.c_int, [C.c_void_p, C.POINTER(SolveStats)]),
    "flipgpu_get_pressure": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "flipgpu_project": (C.c_int, [C.c_void_p, C.POINTER(SolveStats)]),
    "flipgpu_picflip": (C.c_int, [C.c_void_p, C.POINTER(SolveStats)]),
    "flipgpu_advect": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "flipgpu_correct": (C.c_int, [C.c_void_p]),
    "flipgpu_step": (C.c_int, [C.c_void_p, C.POINTER(SolveStats)]),
    "flipgpu_step_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.POINTER(SolveStats)]),
    "flipgpu_launch_count": (C.c_int64, [C.c_void_p]),
    "flipgpu_put_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "flipgpu_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "flipgpu_set_ic_tag_counter": (C.c_int, [C.c_void_p, C.c_uint]),
    "flipgpu_get_ic_tag_counter": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint)]),
    "flipgpu_get_profile": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "flipgpu_get_kernel_profile": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int]),
    "flipgpu_sort_cells_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_void_p]),
    "flipgpu_set_params": (C.c_int, [C.c_void_p, C.POINTER(Params)]),
    "flipgpu_fetch_velocity": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int]),
    "flipgpu_step_async": (C.c_int, [C.c_void_p]),
    "flipgpu_capture_step": (C.c_int, [C.c_void_p]),
    "flipgpu_step_graph": (C.c_int, [C.c_void_p]),
    "flipgpu_last_solve_stats": (C.c_int, [C.c_void_p, C.POINTER(SolveStats)]),
    "flipbatch_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "flipbatch_destroy": (C.c_int, [C.c_void_p]),
    "flipbatch_add": (C.c_int, [C.c_void_p, C.c_void_p]),
    "flipbatch_capture": (C.c_int, [C.c_void_p]),
    "flipbatch_step": (C.c_int, [C.c_void_p]),
    "flipbatch_sync": (C.c_int, [C.c_void_p]),
    "flipbatch_tune": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "flipgpu_set_solve_blocks": (C.c_int, [C.c_void_p, C.c_int]),
    "flipgpu_get_solve_blocks": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "flipunet_param_count": (C.c_int64, []),
    "flipunet_create": (C.c_int, [C.c_uint64, C.POINTER(C.c_void_p)]),
    "flipunet_destroy": (C.c_int, [C.c_void_p]),
    "flipunet_last_error": (C.c_char_p, [C.c_void_p]),
    "flipunet_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "flipunet_set_tensor_path": (C.c_int, [C.c_void_p, C.c_int]),
    "flipunet_set_coarsening": (C.c_int, [C.c_void_p, C.c_int]),
    "flipunet_get_coarsening": (C.c_int, [C.c_void_p]),
    "flipunet_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "flipunet_set_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "flipunet_predict": (C.c_int, [C.c_void_p, C.c_int, C.c_int] + [C.c_void_p] * 5),
    "flipunet_gradients": (C.c_int, [C.c_void_p, C.c_int, C.c_int] + [C.c_void_p] * 5 +
                           [C.POINTER(C.c_double), C.c_void_p]),
    "flipunet_train_step": (C.c_int, [C.c_void_p, C.c_int, C.c_int] + [C.c_void_p] * 5 +
                            [C.c_float, C.POINTER(C.c_double)]),
    "flipgpu_set_warm_start": (C.c_int, [C.c_void_p, C.c_void_p]),
    "flipgpu_set_capture": (C.c_int, [C.c_void_p, C.c_int]),
    "flipgpu_get_solve_system": (C.c_int, [C.c_void_p] + [C.c_void_p] * 6 + [C.c_int]),
    "flipgpu_implicit": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int]),
    "flipgpu_mesh": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "flipgpu_get_mesh": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p]),
    "flipgpu_resample": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_float,
                                   C.c_int]),
}

STAGES = ["sort", "density", "mark_water", "p2g", "divergence", "solve", "gradient",
          "extrapolate", "g2p_flip", "advect", "reposition", "correct"]


def load(path: str | None = None):
    """Load libflipgpu.so (building it if stale). Raises if it cannot."""
    global _lib
    if _lib is None:
        path = path or LIB_PATH
        if not os.path.exists(path):
            _build.build()
        if not os.path.exists(path):
            raise FlipGpuError(f"CUDA library missing: {path}")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def default_params(n: int, max_particles: int, **kw) -> Params:
    p = Params()
    load().flipgpu_default_params(C.byref(p), n, max_particles)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dt):
    return None if a is None else np.ascontiguousarray(a, dtype=dt)


EXPORT_OBJ, EXPORT_SUNFLOW = 1, 2


def set_autotune(on: int):
    """flipgpu_set_autotune: 0 off, 1 on, -1 on and forget decisions."""
    load().flipgpu_set_autotune(int(on))


def autotune_report() -> str:
    lib = load()
    size = lib.flipgpu_autotune_report(None, 0)
    buf = C.create_string_buffer(size + 1)
    lib.flipgpu_autotune_report(buf, size + 1)
    return buf.value.decode()


def write_mesh_files(obj_path, sunflow_path, vertices, normals, faces, wall_thick):
    """exporter::write3D's OBJ and Sunflow scene files for a host mesh
    (either path may be None)."""
    lib = load()
    v = np.ascontiguousarray(vertices, np.float64)
    nv = np.ascontiguousarray(normals, np.float64)
    f = np.ascontiguousarray(faces, np.int32)
    args = (v.ctypes.data, nv.ctypes.data, v.size // 3, f.ctypes.data, f.size // 3,
            float(wall_thick))
    for path, fn in ((obj_path, lib.flipgpu_write_obj), (sunflow_path, lib.flipgpu_write_sunflow)):
        if path is not None and fn(path.encode(), *args) != 0:
            raise FlipGpuError(f"cannot write {path}")


CHECKPOINT_KEYS = ("pos", "vel", "nrm", "type", "visible", "dens", "press", "wall_normal")


def checkpoint_write(path: str, n: int, state: dict):
    """Write the reference's checkpoint layout (flipgpu_checkpoint_write)
    from host arrays: pos/vel/nrm [P,3], type/visible u8 [P] (visible
    optional), dens [P], press [n^3], wall_normal [n^3,4], and the header
    values max_dens, pour_time, pour_pos, pour_rad."""
    lib = load()
    arr = {}
    for k, dt in (("pos", np.float32), ("vel", np.float32), ("nrm", np.float32),
                  ("type", np.uint8), ("visible", np.uint8), ("dens", np.float32),
                  ("press", np.float32), ("wall_normal", np.float32)):
        arr[k] = None if state.get(k) is None else np.ascontiguousarray(state[k], dtype=dt)
    c = Checkpoint()
    c.n, c.count = n, int(arr["type"].shape[0])
    c.max_dens = float(state.get("max_dens", 0.0))
    c.pour_time = int(state.get("pour_time", -1))
    c.pour_pos[:] = [float(v) for v in state.get("pour_pos", (0.0, 0.0))]
    c.pour_rad = float(state.get("pour_rad", 0.0))
    for k in CHECKPOINT_KEYS:
        setattr(c, k, None if arr[k] is None else arr[k].ctypes.data)
    rc = lib.flipgpu_checkpoint_write(path.encode(), C.byref(c))
    if rc != 0:
        raise FlipGpuError(f"checkpoint_write failed: {ERRORS.get(rc, rc)}")


def checkpoint_read(path: str, n: int) -> dict:
    """The content of a reference-layout checkpoint for grid n."""
    lib = load()
    cnt = C.c_int(0)
    rc = lib.flipgpu_checkpoint_count(path.encode(), n, C.byref(cnt))
    if rc != 0:
        raise FlipGpuError(f"not a checkpoint of an n={n} grid: {path}")
    P = cnt.value
    out = {"pos": np.zeros((P, 3), np.float32), "vel": np.zeros((P, 3), np.float32),
           "nrm": np.zeros((P, 3), np.float32), "type": np.zeros(P, np.uint8),
           "visible": np.zeros(P, np.uint8), "dens": np.zeros(P, np.float32),
           "press": np.zeros(n ** 3, np.float32), "wall_normal": np.zeros((n ** 3, 4), np.float32)}
    c = Checkpoint()
    c.n, c.count = n, P
    for k in CHECKPOINT_KEYS:
        setattr(c, k, out[k].ctypes.data)
    rc = lib.flipgpu_checkpoint_read(path.encode(), C.byref(c))
    if rc != 0:
        raise FlipGpuError(f"checkpoint_read failed: {ERRORS.get(rc, rc)}")
    out.update(max_dens=c.max_dens, pour_time=c.pour_time, pour_pos=tuple(c.pour_pos),
               pour_rad=c.pour_rad, count=P)
    return out


class Simulation:
    """One device-resident simulation (a FlipGpu handle)."""

    def __init__(self, params: Params):
        self.lib = load()
        self.params = params
        self.n = params.n
        h = C.c_void_p()
        rc = self.lib.flipgpu_create(C.byref(params), C.byref(h))
        if rc != OK:
            raise FlipGpuError(f"flipgpu_create failed: {ERRORS.get(rc, rc)}")
        self.h = h
        self.np = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.flipgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _ck(self, rc, what):
        if rc != OK:
            msg = self.lib.flipgpu_last_error(self.h)
            raise FlipGpuError(f"{what}: {ERRORS.get(rc, rc)}: {msg.decode() if msg else ''}")
        return rc

    # ------------------------------------------------------------ state
    def set_particles(self, pos, typ, vel=None, nrm=None, dens=None):
        pos = _c(pos, np.float32)
        self.np = pos.shape[0]
        self._keep = [pos, _c(typ, np.uint8), _c(vel, np.float32), _c(nrm, np.float32),
                      _c(dens, np.float32)]
        k = self._keep
        self._ck(self.lib.flipgpu_set_particles(self.h, self.np, _ptr(k[0]), _ptr(k[2]),
                                                _ptr(k[1]), _ptr(k[3]), _ptr(k[4]), 0),
                 "set_particles")

    def set_scene(self, scene):
        self.set_particles(scene.pos, scene.type, scene.vel, scene.nrm)

    def export_mesh(self, directory, frame, wall_thick, formats=3, sunflow_template=None,
                    wait=True):
        """Write the last mesh (after mesh()) as the reference's OBJ and/or
        Sunflow files under directory; asynchronous unless wait."""
        t = None if sunflow_template is None else sunflow_template.encode()
        self._ck(self.lib.flipgpu_export_mesh(self.h, directory.encode(), frame, wall_thick,
                                              formats, t), "export_mesh")
        if wait:
            self._ck(self.lib.flipgpu_export_wait(self.h), "export_wait")

    def preview(self, width=1024, height=700):
        """write_frame's point-splat image: uint8 [height, width, 4]."""
        img = np.zeros((height, width, 4), np.uint8)
        self._ck(self.lib.flipgpu_preview(self.h, img.ctypes.data, width, height, 0), "preview")
        return img

    def write_preview(self, path, width=1024, height=700):
        img = self.preview(width, height)
        if self.lib.flipgpu_write_bmp(path.encode(), img.ctypes.data, width, height) != 0:
            raise FlipGpuError(f"cannot write {path}")
        return img

    def export_wait(self):
        self._ck(self.lib.flipgpu_export_wait(self.h), "export_wait")

    def save_state(self, path, pour_time=-1, pour_pos=(0.0, 0.0), pour_rad=0.12):
        """The reference's checkpoint file of this state (flipgpu_save_state)."""
        pp = (C.c_float * 2)(*pour_pos)
        self._ck(self.lib.flipgpu_save_state(self.h, path.encode(), pour_time, pp, pour_rad),
                 "save_state")

    def load_state(self, path):
        """Replace the state from a reference checkpoint; returns the pour
        settings it carried."""
        t, r = C.c_int(0), C.c_float(0)
        pp = (C.c_float * 2)()
        self._ck(self.lib.flipgpu_load_state(self.h, path.encode(), C.byref(t), pp, C.byref(r)),
                 "load_state")
        self.np = int(self.lib.flipgpu_particle_count(self.h))
        return {"pour_time": t.value, "pour_pos": tuple(pp), "pour_rad": r.value}

    def seed_scene(self, objects, seed=0, density=0.5, jitter=0.25):
        """flipgpu_seed_scene: the particles scenes.build(n, objects, seed,
        density, jitter) makes on the host, generated on the device."""
        from . import scenes as _sc
        arr = (SceneObject * max(len(objects), 1))()
        for o, obj in zip(arr, objects):
            if isinstance(obj, _sc.Box):
                o.shape, o.lo[:], o.hi[:] = 0, obj.lo, obj.hi
            else:
                o.shape, o.c[:], o.r = 1, obj.c, obj.r
            o.vel[:] = obj.vel
        self._ck(self.lib.flipgpu_seed_scene(self.h, arr, len(objects), seed, density, jitter),
                 "seed_scene")
        self.np = int(self.lib.flipgpu_particle_count(self.h))

    def get_particles(self):
        pos = np.zeros((self.np, 3), np.float32)
        vel = np.zeros((self.np, 3), np.float32)
        dens = np.zeros(self.np, np.float32)
        typ = np.zeros(self.np, np.uint8)
        self._ck(self.lib.flipgpu_get_particles(self.h, _ptr(pos), _ptr(vel), _ptr(dens),
                                                _ptr(typ), 0), "get_particles")
        return pos, vel, dens, typ

    def set_grid(self, u=None, A=None, L=None, press=None, div=None):
        u = [None] * 3 if u is None else [_c(x, np.float32) for x in u]
        arrs = u + [_c(A, np.uint8), _c(L, np.float32), _c(press, np.float32),
                    _c(div, np.float32)]
        self._ck(self.lib.flipgpu_set_grid(self.h, *[_ptr(a) for a in arrs], 0), "set_grid")

    def get_grid(self):
        n = self.n
        nf = (n + 1) * n * n
        u = [np.zeros(nf, np.float32) for _ in range(3)]
        A = np.zeros(n ** 3, np.uint8)
        L = np.zeros(n ** 3, np.float32)
        p = np.zeros(n ** 3, np.float32)
        d = np.zeros(n ** 3, np.float32)
        self._ck(self.lib.flipgpu_get_grid(self.h, *[_ptr(a) for a in (*u, A, L, p, d)], 0),
                 "get_grid")
        return u, A, L, p, d

    def get_cells(self):
        cs = np.zeros(self.n ** 3 + 1, np.uint32)
        perm = np.zeros(self.np, np.uint32)
        self._ck(self.lib.flipgpu_get_cells(self.h, _ptr(cs), _ptr(perm), 0), "get_cells")
        return cs, perm

    def set_max_density(self, md):
        self._ck(self.lib.flipgpu_set_max_density(self.h, C.c_float(md)), "set_max_density")

    def calibrate_max_density(self):
        out = C.c_float(0)
        self._ck(self.lib.flipgpu_calibrate_max_density(self.h, C.byref(out)), "calibrate")
        return out.value

    def set_step(self, step):
        self._ck(self.lib.flipgpu_set_step(self.h, step), "set_step")

    def set_stream(self, stream_handle):
        """Launch on an external cudaStream_t (an integer handle); None restores
        the handle's own stream."""
        self._ck(self.lib.flipgpu_set_stream(self.h, C.c_void_p(stream_handle)), "set_stream")

    def sync(self):
        self._ck(self.lib.flipgpu_sync(self.h), "sync")

    def put_state(self, pos, vel, on_device=False):
        """pos/vel: numpy arrays (host) or raw device addresses (on_device)."""
        if on_device:
            self._ck(self.lib.flipgpu_put_state(self.h, C.c_void_p(pos), C.c_void_p(vel), 1),
                     "put_state")
        else:
            self._ck(self.lib.flipgpu_put_state(self.h, _ptr(pos), _ptr(vel), 0), "put_state")

    def get_state_into(self, pos_ptr, vel_ptr):
        """Download positions/velocities into host buffers given by address."""
        self._ck(self.lib.flipgpu_get_particles(self.h, C.c_void_p(pos_ptr),
                                                C.c_void_p(vel_ptr), None, None, 0),
                 "get_particles")

    def fetch_velocity(self, pts):
        """mapper::fetchVelocity at each point of pts [m,3]."""
        pts = _c(pts, np.float32)
        out = np.zeros_like(pts)
        self._ck(self.lib.flipgpu_fetch_velocity(self.h, pts.shape[0], _ptr(pts), _ptr(out), 0),
                 "fetch_velocity")
        return out

    def resample(self, pts, vel, re):
        """corrector::resample at each point (vel: fallback values)."""
        pts = _c(pts, np.float32)
        out = _c(vel, np.float32).copy()
        self._ck(self.lib.flipgpu_resample(self.h, pts.shape[0], _ptr(pts), _ptr(out),
                                           C.c_float(re), 0), "resample")
        return out

    def solve_blocks(self, value=None) -> int:
        """The cap on the persistent solve's grid (0 = none); sets it first
        when value is given."""
        if value is not None:
            self._ck(self.lib.flipgpu_set_solve_blocks(self.h, int(value)), "set_solve_blocks")
        out = C.c_int()
        self._ck(self.lib.flipgpu_get_solve_blocks(self.h, C.byref(out)), "get_solve_blocks")
        return out.value

    def ic_tag_counter(self, value=None):
        """The IC wavefront's tag counter (a testing aid): set it when value
        is given; returns the current value."""
        if value is not None:
            self._ck(self.lib.flipgpu_set_ic_tag_counter(self.h, int(value)), "set_ic_tag_counter")
        out = C.c_uint(0)
        self._ck(self.lib.flipgpu_get_ic_tag_counter(self.h, C.byref(out)), "get_ic_tag_counter")
        return out.value

    def set_profiling(self, on=True):
        self._ck(self.lib.flipgpu_set_profiling(self.h, int(on)), "set_profiling")

    def profile(self):
        ms = np.zeros(len(STAGES), np.float64)
        calls = np.zeros(len(STAGES), np.int64)
        self._ck(self.lib.flipgpu_get_profile(self.h, _ptr(ms), _ptr(calls), len(STAGES)),
                 "get_profile")
        return {s: (float(ms[i]), int(calls[i])) for i, s in enumerate(STAGES)}

    def kernel_profile(self):
        """{kernel: (ms, launches)} of the main kernels since profiling was
        switched on (flipgpu_get_kernel_profile)."""
        size = self.lib.flipgpu_get_kernel_profile(self.h, None, 0)
        if size < 0:
            raise FlipGpuError(f"get_kernel_profile failed ({size})")
        buf = C.create_string_buffer(size + 1)
        self.lib.flipgpu_get_kernel_profile(self.h, buf, size + 1)
        out = {}
        for line in buf.value.decode().splitlines():
            name, ms, calls = line.split("\t")
            out[name] = (float(ms), int(calls))
        return out

    @property
    def launches(self):
        return self.lib.flipgpu_launch_count(self.h)

    # ----------------------------------------------------------- stages
    def sort(self):
        self._ck(self.lib.flipgpu_sort(self.h), "sort")

    def compute_density(self):
        self._ck(self.lib.flipgpu_compute_density(self.h), "compute_density")

    def mark_water(self):
        self._ck(self.lib.flipgpu_mark_water(self.h), "mark_water")

    def add_force(self):
        self._ck(self.lib.flipgpu_add_force(self.h), "add_force")

    def p2g(self):
        self._ck(self.lib.flipgpu_p2g(self.h), "p2g")

    def g2p(self):
        self._ck(self.lib.flipgpu_g2p(self.h), "g2p")

    def _stats_call(self, fn, what):
        st = SolveStats()
        self._ck(fn(self.h, C.byref(st)), what)
        return st

    def implicit(self, pts):
        """implicit::implicit_func at each point of pts [m,3] (float64)."""
        pts = _c(pts, np.float32)
        out = np.zeros(pts.shape[0], np.float64)
        self._ck(self.lib.flipgpu_implicit(self.h, pts.shape[0], _ptr(pts), _ptr(out), 0),
                 "implicit")
        return out

    def set_params(self, params: Params):
        """Change run parameters (n and max_particles must stay)."""
        self._ck(self.lib.flipgpu_set_params(self.h, C.byref(params)), "set_params")
        self.params = params

    def step_async(self):
        """One step with no host synchronisation (FAST solver)."""
        self._ck(self.lib.flipgpu_step_async(self.h), "step_async")

    def capture_step(self):
        """Record one step as a CUDA graph; step_graph replays it."""
        self._ck(self.lib.flipgpu_capture_step(self.h), "capture_step")

    def step_graph(self):
        self._ck(self.lib.flipgpu_step_graph(self.h), "step_graph")

    def last_solve_stats(self):
        st = SolveStats()
        self._ck(self.lib.flipgpu_last_solve_stats(self.h, C.byref(st)), "last_solve_stats")
        return st

    def set_warm_start(self, net):
        """Attach a UNet (or None) to this simulation's FAST-mode solves."""
        self._warm = net
        self._ck(self.lib.flipgpu_set_warm_start(self.h, net.h if net is not None else None),
                 "set_warm_start")

    def set_capture(self, on=True):
        self._ck(self.lib.flipgpu_set_capture(self.h, 1 if on else 0), "set_capture")

    def solve_system(self, dev=None):
        """The last solve's (A, L, b, x0, r0, x): numpy arrays, or copies into
        the device buffers dev = (A, L, b, x0, r0, x) given as raw addresses
        (None skips one)."""
        if dev is not None:
            self._ck(self.lib.flipgpu_get_solve_system(
                self.h, *[C.c_void_p(a) if a is not None else None for a in dev], 1),
                "get_solve_system")
            return None
        nc = self.n ** 3
        A = np.zeros(nc, np.uint8)
        L, b, x0, r0, x = (np.zeros(nc, np.float32) for _ in range(5))
        self._ck(self.lib.flipgpu_get_solve_system(self.h, _ptr(A), _ptr(L), _ptr(b), _ptr(x0),
                                                   _ptr(r0), _ptr(x), 0), "get_solve_system")
        return A, L, b, x0, r0, x

    def mesh_counts(self):
        """Build the mesh on the device only; returns (vertices, faces)."""
        nv, nf = C.c_int64(), C.c_int64()
        self._ck(self.lib.flipgpu_mesh(self.h, C.byref(nv), C.byref(nf)), "mesh")
        return nv.value, nf.value

    def mesh(self, field=False):
        """mesher::generateMesh on the lists of the last sort: dict of
        vertices, normals (float64 [nv,3]), faces (int32 [nf,3]) and, with
        field=True, the meshed field ((n+1)^3 float32, x fastest)."""
        nv, nf = C.c_int64(), C.c_int64()
        self._ck(self.lib.flipgpu_mesh(self.h, C.byref(nv), C.byref(nf)), "mesh")
        out = {"vertices": np.zeros((nv.value, 3), np.float64),
               "normals": np.zeros((nv.value, 3), np.float64),
               "faces": np.zeros((nf.value, 3), np.int32)}
        if field:
            out["field"] = np.zeros((self.n + 1) ** 3, np.float32)
        self._ck(self.lib.flipgpu_get_mesh(self.h, _ptr(out["vertices"]), _ptr(out["normals"]),
                                           _ptr(out["faces"]),
                                           _ptr(out["field"]) if field else None), "get_mesh")
        return out

    def solve(self):
        return self._stats_call(self.lib.flipgpu_solve, "solve")

    def get_pressure(self):
        """The last solve's pressure as float64 [n^3]: the double-float
        iterate of a refined FAST solve, else the FP32 pressure grid."""
        out = np.zeros(self.n ** 3, np.float64)
        self._ck(self.lib.flipgpu_get_pressure(self.h, _ptr(out), 0), "get_pressure")
        return out

    def project(self):
        return self._stats_call(self.lib.flipgpu_project, "project")

    def picflip(self):
        return self._stats_call(self.lib.flipgpu_picflip, "picflip")

    def advect(self, want_stuck=True):
        s = C.c_int(0)
        self._ck(self.lib.flipgpu_advect(self.h, C.byref(s) if want_stuck else None), "advect")
        return s.value

    def correct(self):
        self._ck(self.lib.flipgpu_correct(self.h), "correct")

    def step(self):
        return self._stats_call(self.lib.flipgpu_step, "step")

    def step_host(self, pos_in=None, vel_in=None, pos_out=None, vel_out=None):
        """One step on host AoS float[np][3] buffers (numpy arrays, ideally
        views of pinned memory; in and out may be the same arrays): upload,
        step and download with the transfers overlapped with the step."""
        def addr(a, writable):
            if a is None:
                return None
            if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and
                    a.flags["C_CONTIGUOUS"] and a.size == 3 * self.np):
                raise ValueError("step_host wants contiguous float32 arrays of np x 3")
            if writable and not a.flags["WRITEABLE"]:
                raise ValueError("step_host output arrays must be writable")
            return C.c_void_p(a.ctypes.data)
        st = SolveStats()
        self._ck(self.lib.flipgpu_step_host(self.h, addr(pos_in, False), addr(vel_in, False),
                                            addr(pos_out, True), addr(vel_out, True),
                                            C.byref(st)), "step_host")
        return st


class UNet:
    """The learned warm start's network (libflipgpu's flipunet_* calls).
    Array arguments of predict/gradients/train_step are raw device addresses
    (e.g. torch tensors' data_ptr()) of batch systems of n^3 cells."""

    def __init__(self, seed=0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.flipunet_create(seed, C.byref(h))
        if rc != 0:
            raise FlipGpuError(f"flipunet_create failed ({rc})")
        self.h = h
        self.nparam = int(self.lib.flipunet_param_count())

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.flipunet_destroy(self.h)
            self.h = None

    def _ck(self, rc, what):
        if rc != 0:
            msg = self.lib.flipunet_last_error(self.h)
            raise FlipGpuError(f"{what}: {msg.decode() if msg else rc}")

    def set_stream(self, stream_handle):
        self._ck(self.lib.flipunet_set_stream(self.h, C.c_void_p(stream_handle)), "set_stream")

    def set_coarsening(self, levels: int):
        """Run the network on the grid pooled `levels` times (0..3) and
        prolong its output trilinearly to the solver's grid."""
        self._ck(self.lib.flipunet_set_coarsening(self.h, int(levels)), "set_coarsening")

    @property
    def coarsening(self) -> int:
        return int(self.lib.flipunet_get_coarsening(self.h))

    def set_tensor_path(self, tcgen05: bool):
        """Forward convolutions on tcgen05 (True, the default) or mma.sync."""
        self._ck(self.lib.flipunet_set_tensor_path(self.h, 1 if tcgen05 else 0), "set_tensor_path")

    def params(self):
        p = np.zeros(self.nparam, np.float32)
        self._ck(self.lib.flipunet_get_params(self.h, _ptr(p)), "get_params")
        return p

    def set_params(self, p):
        p = _c(p, np.float32)
        assert p.shape[0] == self.nparam
        self._ck(self.lib.flipunet_set_params(self.h, _ptr(p)), "set_params")

    def save(self, path, **meta):
        """Parameters as raw float32; the coarsening (and any extra keys)
        in a JSON file beside them."""
        self.params().tofile(path)
        with open(path + ".json", "w") as f:
            json.dump({"coarsening": self.coarsening, **meta}, f)

    def load(self, path):
        self.set_params(np.fromfile(path, np.float32))
        if os.path.exists(path + ".json"):
            with open(path + ".json") as f:
                self.set_coarsening(int(json.load(f).get("coarsening", 0)))

    def predict(self, n, batch, A, b, x0, r0, delta):
        self._ck(self.lib.flipunet_predict(self.h, n, batch, *[C.c_void_p(a) for a in
                                                             (A, b, x0, r0, delta)]), "predict")

    def gradients(self, n, batch, A, b, x0, r0, x):
        loss = C.c_double()
        g = np.zeros(self.nparam, np.float32)
        self._ck(self.lib.flipunet_gradients(self.h, n, batch,
                                             *[C.c_void_p(a) for a in (A, b, x0, r0, x)],
                                             C.byref(loss), _ptr(g)), "gradients")
        return loss.value, g

    def train_step(self, n, batch, A, b, x0, r0, x, lr):
        loss = C.c_double()
        self._ck(self.lib.flipunet_train_step(self.h, n, batch,
                                              *[C.c_void_p(a) for a in (A, b, x0, r0, x)],
                                              C.c_float(lr), C.byref(loss)), "train_step")
        return loss.value


class Batch:
    """Independent simulations advanced together (flipbatch_*): every
    member's step runs on its own stream without host waits, optionally
    replayed from CUDA graphs."""

    def __init__(self, sims=()):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.flipbatch_create(C.byref(h))
        if rc != OK:
            raise FlipGpuError(f"flipbatch_create failed ({rc})")
        self.h = h
        self.sims = []
        for s in sims:
            self.add(s)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.flipbatch_destroy(self.h)
            self.h = None

    def _ck(self, rc, what):
        if rc != OK:
            errs = [s.lib.flipgpu_last_error(s.h).decode() for s in self.sims]
            raise FlipGpuError(f"{what} failed ({rc}): {[e for e in errs if e][:3]}")

    def add(self, sim):
        self._ck(self.lib.flipbatch_add(self.h, sim.h), "add")
        self.sims.append(sim)

    def capture(self):
        self._ck(self.lib.flipbatch_capture(self.h), "capture")

    def step(self):
        self._ck(self.lib.flipbatch_step(self.h), "step")

    def sync(self):
        self._ck(self.lib.flipbatch_sync(self.h), "sync")

    def tune(self) -> float:
        """Share the GPU between the members' solves (flipbatch_tune): the
        chosen share, 0.0 for uncapped grids. The members must have stepped."""
        out = C.c_double()
        self._ck(self.lib.flipbatch_tune(self.h, C.byref(out)), "tune")
        return out.value

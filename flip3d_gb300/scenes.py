"""Scene setup for the FLIP step: seeded particle sets on the unit cube.

This is host-side initialisation, run once per simulation, standing in for the
reference's ``flip3D::init`` (src/flip3D.cpp:649-777):

* walls: the six 1-cell boxes of ``placeWalls`` (src/flip3D.cpp:300-362), one
  wall particle at the centre of every wall cell (src/flip3D.cpp:729-740),
  with the face normals of ``compute_wall_normal`` (src/flip3D.cpp:75-130);
* liquid: a lattice of spacing DENSITY cells (2x2x2 per cell) filtered to the
  interior and to the liquid objects, first matching object wins as in
  ``pushParticle`` (src/flip3D.cpp:580-647). Each particle is jittered by a
  uniform +-0.25 cell per axis from the counter-based generator of
  include/flip_rng.h (the reference jitters by +-0.002 cell with rand());
* the order of the particle vector is the reference's: liquid in lattice order
  (i outer, k inner), then walls in cell order.

The scenes are those the benchmark configurations name: a pool plus a sphere,
a dam-break column, a sphere falling into a pool, and random multi-object
scenes for the learned warm start.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

FLUID = 1
WALL = 2

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_GOLD = np.uint64(0x9E3779B97F4A7C15)
_BKEY = np.uint64(0x632BE59BD9B4E019)
RNG_SEED = 1


def _mix64(z: np.ndarray) -> np.ndarray:
    z = z ^ (z >> np.uint64(30))
    z = z * _M1
    z = z ^ (z >> np.uint64(27))
    z = z * _M2
    z = z ^ (z >> np.uint64(31))
    return z


def flip_stream(use: int, step: int, comp: int) -> int:
    return ((use & 0xFF) << 56) | ((step & 0xFFFFFFFFFF) << 8) | (comp & 0xFF)


def flip_rand31(seed: int, stream: int, a, b=0) -> np.ndarray:
    """Vectorised include/flip_rng.h:flip_rand31 over index array ``a``."""
    with np.errstate(over="ignore"):
        h = _mix64(np.uint64(seed) ^ _GOLD)
        h = _mix64(h ^ np.uint64(stream))
        h = _mix64(h + np.asarray(a, dtype=np.uint64))
        h = _mix64(h + (np.asarray(b, dtype=np.uint64) ^ _BKEY))
    return (h >> np.uint64(33)).astype(np.uint32)


@dataclass
class Box:
    lo: tuple
    hi: tuple
    vel: tuple = (0.0, 0.0, 0.0)


@dataclass
class Sphere:
    c: tuple
    r: float
    vel: tuple = (0.0, 0.0, 0.0)


@dataclass
class Scene:
    n: int
    pos: np.ndarray  # float32 [P,3]
    vel: np.ndarray  # float32 [P,3]
    type: np.ndarray  # uint8 [P]
    nrm: np.ndarray  # float32 [P,3]
    name: str = ""
    objects: list = field(default_factory=list)

    @property
    def count(self) -> int:
        return int(self.type.shape[0])

    @property
    def fluid_count(self) -> int:
        return int((self.type == FLUID).sum())


def _inside(obj, x, y, z, n):
    if isinstance(obj, Box):
        lo = np.float32(obj.lo[0]), np.float32(obj.lo[1]), np.float32(obj.lo[2])
        hi = np.float32(obj.hi[0]), np.float32(obj.hi[1]), np.float32(obj.hi[2])
        return ((x > lo[0]) & (x < hi[0]) & (y > lo[1]) & (y < hi[1]) &
                (z > lo[2]) & (z < hi[2]))
    px = x.astype(np.float32)
    py = y.astype(np.float32)
    pz = z.astype(np.float32)
    c = np.float32(obj.c[0]), np.float32(obj.c[1]), np.float32(obj.c[2])
    ln = np.hypot(np.hypot(px - c[0], py - c[1]), pz - c[2])
    return ln < np.float32(obj.r)


def build(n: int, objects: list, seed: int = 0, density: float = 0.5,
          jitter: float = 0.25, name: str = "") -> Scene:
    """Seed the liquid ``objects`` and the cube walls on an n^3 grid."""
    wall = 1.0 / n
    w = density * wall
    m = int(round(n / density))
    idx = (np.arange(m, dtype=np.float64) * w + w / 2.0)
    interior = (idx > wall) & (idx < 1.0 - wall)
    ii = np.nonzero(interior)[0]
    pos_chunks, vel_chunks = [], []
    lat = np.arange(m, dtype=np.int64)
    for i in ii:
        x = idx[i]
        jj, kk = np.meshgrid(ii, ii, indexing="ij")
        jj = jj.ravel()
        kk = kk.ravel()
        y = idx[jj]
        z = idx[kk]
        xs = np.full_like(y, x)
        owner = np.full(y.shape, -1, dtype=np.int32)
        for oi, obj in enumerate(objects):
            hit = _inside(obj, xs, y, z, n) & (owner < 0)
            owner[hit] = oi
        sel = owner >= 0
        if not sel.any():
            continue
        jj, kk, owner = jj[sel], kk[sel], owner[sel]
        lattice_index = ((np.int64(i) * m + lat[jj]) * m + lat[kk]).astype(np.uint64)
        p = np.empty((jj.size, 3), dtype=np.float64)
        p[:, 0] = x
        p[:, 1] = idx[jj]
        p[:, 2] = idx[kk]
        for c in range(3):
            r = flip_rand31(seed, flip_stream(RNG_SEED, 0, c), lattice_index)
            u01 = r.astype(np.float64) / 2147483648.0
            p[:, c] += (u01 - 0.5) * 2.0 * jitter * wall
        pos_chunks.append(p.astype(np.float32))
        v = np.array([objects[o].vel for o in range(len(objects))],
                     dtype=np.float32)[owner]
        vel_chunks.append(v)
    fpos = np.concatenate(pos_chunks) if pos_chunks else np.zeros((0, 3), np.float32)
    fvel = np.concatenate(vel_chunks) if vel_chunks else np.zeros((0, 3), np.float32)

    # Wall particles at wall-cell centres, in cell order (src/flip3D.cpp:729-740).
    c = (np.arange(n, dtype=np.float64) * wall + wall / 2.0)
    gi, gj, gk = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    onwall = ((gi == 0) | (gi == n - 1) | (gj == 0) | (gj == n - 1) |
              (gk == 0) | (gk == n - 1)).ravel()
    wpos = np.stack([c[gi.ravel()[onwall]], c[gj.ravel()[onwall]],
                     c[gk.ravel()[onwall]]], axis=1).astype(np.float32)
    # compute_wall_normal for cube walls (src/flip3D.cpp:87-129).
    wn = np.zeros_like(wpos)
    lo = np.float64(1.1 * wall)
    hi = np.float64(1.0 - 1.1 * wall)
    for a in range(3):
        wn[:, a] += np.where(wpos[:, a].astype(np.float64) <= lo, 1.0, 0.0)
        wn[:, a] = np.where(wpos[:, a].astype(np.float64) >= hi, -1.0, wn[:, a])
    d = np.hypot(np.hypot(wn[:, 0], wn[:, 1]), wn[:, 2]).astype(np.float32)
    nz = d != 0
    wn[nz] = wn[nz] / d[nz, None]

    # Fluid particles that landed in a wall cell are erased
    # (src/flip3D.cpp:742-761); the walls are the outer cell layer.
    if fpos.shape[0]:
        cell = np.clip((np.float32(n) * fpos).astype(np.float64), 0, n - 1).astype(np.int64)
        keep = ~((cell == 0) | (cell == n - 1)).any(axis=1)
        fpos, fvel = fpos[keep], fvel[keep]

    pos = np.concatenate([fpos, wpos]).astype(np.float32)
    vel = np.concatenate([fvel, np.zeros_like(wpos)]).astype(np.float32)
    typ = np.concatenate([np.full(fpos.shape[0], FLUID, np.uint8),
                          np.full(wpos.shape[0], WALL, np.uint8)])
    nrm = np.concatenate([np.zeros_like(fpos), wn]).astype(np.float32)
    return Scene(n=n, pos=np.ascontiguousarray(pos), vel=np.ascontiguousarray(vel),
                 type=typ, nrm=np.ascontiguousarray(nrm), name=name,
                 objects=list(objects))


def pool_sphere(n: int = 32, seed: int = 0) -> Scene:
    """Pool y<0.3 plus a sphere r=0.15 at (0.5,0.7,0.5), at rest."""
    wall = 1.0 / n
    return build(n, [Box((wall, wall, wall), (1 - wall, 0.3, 1 - wall)),
                     Sphere((0.5, 0.7, 0.5), 0.15)], seed, name=f"pool_sphere_n{n}")


def dam_break(n: int = 128, seed: int = 0) -> Scene:
    """Liquid column x<0.4, y<0.8, full z, at rest."""
    wall = 1.0 / n
    return build(n, [Box((wall, wall, wall), (0.4, 0.8, 1 - wall))], seed,
                 name=f"dam_break_n{n}")


def sphere_into_pool(n: int = 256, seed: int = 0) -> Scene:
    """Pool of depth 0.25 and a sphere r=0.15 at (0.5,0.75,0.5) moving (0,-2,0)."""
    wall = 1.0 / n
    return build(n, [Box((wall, wall, wall), (1 - wall, 0.25, 1 - wall)),
                     Sphere((0.5, 0.75, 0.5), 0.15, (0.0, -2.0, 0.0))], seed,
                 name=f"sphere_into_pool_n{n}")


def random_scene(n: int, seed: int) -> Scene:
    """1-4 liquid boxes/spheres (size 0.1-0.3), pool depth U(0,0.4),
    initial velocities N(0,1) m/s."""
    rng = np.random.default_rng(seed)
    wall = 1.0 / n
    objs = []
    depth = rng.uniform(0.0, 0.4)
    if depth > 1.5 * wall:
        objs.append(Box((wall, wall, wall), (1 - wall, depth, 1 - wall)))
    for _ in range(int(rng.integers(1, 5))):
        size = rng.uniform(0.1, 0.3)
        c = rng.uniform(0.2, 0.8, size=3)
        v = tuple(float(x) for x in rng.normal(0.0, 1.0, size=3))
        if rng.random() < 0.5:
            objs.append(Sphere(tuple(float(x) for x in c), size / 2.0, v))
        else:
            lo = tuple(float(max(wall, x - size / 2)) for x in c)
            hi = tuple(float(min(1 - wall, x + size / 2)) for x in c)
            objs.append(Box(lo, hi, v))
    return build(n, objs, seed, name=f"random_n{n}_s{seed}")


BATCH_SIZES = (24, 32, 48, 64, 96)


def batch_scene(seed: int) -> Scene:
    """One scene of the batched workload: N uniform from {24,32,48,64,96},
    pool depth U(0.1, 0.4), a sphere of radius U(0.08, 0.2) above it (falling
    from rest)."""
    rng = np.random.default_rng(seed)
    n = int(rng.choice(BATCH_SIZES))
    wall = 1.0 / n
    depth = float(rng.uniform(0.1, 0.4))
    r = float(rng.uniform(0.08, 0.2))
    cx, cz = (float(v) for v in rng.uniform(0.2 + r / 2, 0.8 - r / 2, size=2))
    cy = float(min(1.0 - wall - r - 0.02, depth + r + rng.uniform(0.05, 0.3)))
    return build(n, [Box((wall, wall, wall), (1 - wall, depth, 1 - wall)),
                     Sphere((cx, cy, cz), r)], seed, name=f"batch_s{seed}_n{n}")


def calibration_lattice(n: int, density: float = 0.5) -> np.ndarray:
    """The 10^3 lattice whose peak density normalises ``dens``
    (src/flip3D.cpp:689-699)."""
    h = np.float32(density / n)
    i, j, k = np.meshgrid(np.arange(10), np.arange(10), np.arange(10), indexing="ij")
    pos = np.stack([(i.ravel() + 0.5) * np.float64(h), (j.ravel() + 0.5) * np.float64(h),
                    (k.ravel() + 0.5) * np.float64(h)], axis=1)
    return pos.astype(np.float32)


SCENES = {
    "pool_sphere": pool_sphere,
    "dam_break": dam_break,
    "sphere_into_pool": sphere_into_pool,
}

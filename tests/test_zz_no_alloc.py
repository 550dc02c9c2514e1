"""flipgpu_sort_cells_noalloc: the cell sort for callers that may not allocate
device memory (a plugin whose host application owns the GPU's memory, a frame
loop that cannot stall on cudaMalloc/cudaFree). It must produce exactly the
cell lists of the allocating entry point, flipgpu_sort, and do so on
consecutive calls that reuse its fixed scratch array. The test allocates its
own device buffers with torch; the entry point itself allocates nothing.

This file sorts last so that a run stopping at the first failure has run
every other test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from flip3d_gb300 import scenes

pytestmark = pytest.mark.gpu


def reference_cells(gpu, sc):
    sim = gpu.Simulation(gpu.default_params(sc.n, sc.count))
    sim.set_scene(sc)
    sim.sort()
    cs, perm = sim.get_cells()
    sim.close()
    return cs, perm


def noalloc_cells(gpu, torch, sc, n=None, pos=None):
    lib = gpu.load()
    dev = torch.device("cuda", 0)
    n = sc.n if n is None else n
    pos = sc.pos if pos is None else pos
    count = len(pos)
    pos_d = torch.from_numpy(np.ascontiguousarray(pos, dtype=np.float32).reshape(-1)).to(dev)
    cs = torch.full((n ** 3 + 1,), -1, dtype=torch.int32, device=dev)
    perm = torch.full((max(count, 1),), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.flipgpu_sort_cells_noalloc(n, count, C.c_void_p(pos_d.data_ptr()),
                                        C.c_void_p(cs.data_ptr()), C.c_void_p(perm.data_ptr()),
                                        C.c_void_p(stream.cuda_stream))
    assert rc == 0, gpu.ERRORS.get(rc, rc)
    torch.cuda.synchronize()
    return (cs.cpu().numpy().view(np.uint32).copy(),
            perm.cpu().numpy().view(np.uint32)[:count].copy())


def host_cells(n, pos):
    """The reference's cell lists on the host: cell of fmax(0, fmin(n-1, n*p))
    per axis (src/sorter.cpp:35-37), particles in index order within a cell."""
    fn = np.float32(n)
    ijk = np.fmax(np.float32(0), np.fmin(np.float32(n - 1), fn * pos.astype(np.float32)))
    ijk = ijk.astype(np.int64)
    key = (ijk[:, 0] * n + ijk[:, 1]) * n + ijk[:, 2]
    perm = np.argsort(key, kind="stable").astype(np.uint32)
    cs = np.zeros(n ** 3 + 1, np.uint32)
    cs[1:] = np.cumsum(np.bincount(key, minlength=n ** 3))
    return cs, perm


def test_noalloc_sort_matches_allocating_sort_twice():
    torch = pytest.importorskip("torch")
    from flip3d_gb300 import gpu
    # two calls in a row with different inputs: the second must not see the
    # first one's counters
    first = scenes.pool_sphere(32, seed=4)
    second = scenes.dam_break(24, seed=9)
    second.pos[::7] += np.float32(0.3 / 24)  # crowd some cells
    for sc in (first, second):
        want_cs, want_perm = reference_cells(gpu, sc)
        got_cs, got_perm = noalloc_cells(gpu, torch, sc)
        assert np.array_equal(got_cs, want_cs)
        assert np.array_equal(got_perm, want_perm)


def test_noalloc_sort_crowded_and_out_of_range_positions():
    """A crowded cell (2^16 particles clamped into one corner, more than the
    per-thread ordering handles), positions outside the unit cube and
    non-finite ones (clamped as the reference clamps), and many cells just
    above the crowded threshold; compared with the allocating sort and with
    a stable host sort of the same keys."""
    torch = pytest.importorskip("torch")
    from flip3d_gb300 import gpu
    rng = np.random.default_rng(11)
    n = 16
    base = scenes.pool_sphere(n, seed=2)
    crowd = rng.uniform(-0.5, 0.01, size=(1 << 16, 3)).astype(np.float32)  # all in cell 0
    wild = rng.uniform(-3.0, 4.0, size=(5000, 3)).astype(np.float32)
    wild[:8] = [[np.inf, 0.5, 0.5], [-np.inf, 0.5, 0.5], [np.nan, 0.2, 0.9], [0.5, np.nan, 0.5],
                [1.0, 1.0, 1.0], [0.0, 0.0, 0.0], [2.0, -1.0, 0.5], [0.999, 1e30, -1e30]]
    # 40 particles in each of 200 cells: just above the per-thread limit
    cells = rng.choice(n ** 3, size=200, replace=False)
    ci = np.stack([cells // (n * n), (cells // n) % n, cells % n], axis=1)
    centre = ((ci + 0.5) / n).astype(np.float32)
    forty = np.repeat(centre, 40, axis=0) + rng.uniform(-0.4 / n, 0.4 / n, (8000, 3)).astype(
        np.float32)
    pos = np.concatenate([base.pos, crowd, wild, forty]).astype(np.float32)
    pos = pos[rng.permutation(len(pos))]
    typ = np.ones(len(pos), np.uint8)
    want_cs, want_perm = host_cells(n, pos)
    assert want_cs[1] - want_cs[0] >= 1 << 16
    got_cs, got_perm = noalloc_cells(gpu, torch, None, n=n, pos=pos)
    assert np.array_equal(got_cs, want_cs)
    assert np.array_equal(got_perm, want_perm)
    sim = gpu.Simulation(gpu.default_params(n, len(pos)))
    sim.set_particles(pos, typ)
    sim.sort()
    ref_cs, ref_perm = sim.get_cells()
    sim.close()
    assert np.array_equal(got_cs, ref_cs)
    assert np.array_equal(got_perm, ref_perm)


def test_noalloc_sort_empty_input_and_largest_grid():
    torch = pytest.importorskip("torch")
    from flip3d_gb300 import gpu
    cs, perm = noalloc_cells(gpu, torch, None, n=8, pos=np.zeros((0, 3), np.float32))
    assert perm.size == 0 and not cs.any()
    sc = scenes.pool_sphere(64, seed=5)
    pos = sc.pos[: 200_000]
    want_cs, want_perm = host_cells(64, pos)
    got_cs, got_perm = noalloc_cells(gpu, torch, None, n=64, pos=pos)
    assert np.array_equal(got_cs, want_cs)
    assert np.array_equal(got_perm, want_perm)


def test_noalloc_sort_rejects_oversize():
    from flip3d_gb300 import gpu
    lib = gpu.load()
    one = C.c_void_p(1)
    assert lib.flipgpu_sort_cells_noalloc(65, 10, one, one, one, None) == -7
    # n^3 of these wraps in 64 bits; the grid size itself is checked
    assert lib.flipgpu_sort_cells_noalloc(1 << 22, 10, one, one, one, None) == -7
    assert lib.flipgpu_sort_cells_noalloc((1 << 31) - 1, 10, one, one, one, None) == -7
    assert lib.flipgpu_sort_cells_noalloc(16, (1 << 20) + 1, one, one, one, None) == -7
    assert lib.flipgpu_sort_cells_noalloc(0, 10, one, one, one, None) == -1

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


def noalloc_cells(gpu, torch, sc):
    lib = gpu.load()
    dev = torch.device("cuda", 0)
    pos = torch.from_numpy(np.ascontiguousarray(sc.pos)).to(dev)
    cs = torch.full((sc.n ** 3 + 1,), -1, dtype=torch.int32, device=dev)
    perm = torch.full((sc.count,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.flipgpu_sort_cells_noalloc(sc.n, sc.count, C.c_void_p(pos.data_ptr()),
                                        C.c_void_p(cs.data_ptr()), C.c_void_p(perm.data_ptr()),
                                        C.c_void_p(stream.cuda_stream))
    assert rc == 0, gpu.ERRORS.get(rc, rc)
    torch.cuda.synchronize()
    return (cs.cpu().numpy().view(np.uint32).copy(), perm.cpu().numpy().view(np.uint32).copy())


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


def test_noalloc_sort_rejects_oversize():
    from flip3d_gb300 import gpu
    lib = gpu.load()
    one = C.c_void_p(1)
    assert lib.flipgpu_sort_cells_noalloc(65, 10, one, one, one, None) == -7
    assert lib.flipgpu_sort_cells_noalloc(16, (1 << 20) + 1, one, one, one, None) == -7

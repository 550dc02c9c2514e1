"""The byte model behind bench.py's roofline line (host logic only)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_liquid_chunk_cells_counts_128_cell_chunks_with_liquid():
    n = 16  # 4096 cells = 32 chunks of 128
    A = np.zeros(n ** 3, np.uint8)
    assert bench.liquid_chunk_cells(A) == 0
    A[5] = 1          # chunk 0
    A[127] = 1        # chunk 0 again
    A[128 * 7] = 1    # chunk 7
    A[128 * 9] = 2    # a wall cell does not count
    assert bench.liquid_chunk_cells(A) == 2 * 128


def test_mg_coarse_cells():
    assert bench.mg_coarse_cells(128) == 64 ** 3 + 32 ** 3 + 16 ** 3 + 8 ** 3 + 4 ** 3
    assert bench.mg_coarse_cells(48) == 24 ** 3 + 12 ** 3 + 6 ** 3 + 3 ** 3


def test_solve_bytes_per_preconditioner():
    n, iters, cells = 128, 10, 657280
    C = n ** 3
    jac = bench.stage_bytes("solve", 0, n, iters, cells, "jacobi")
    assert jac == 21 * C + iters * 49 * cells
    mg = bench.stage_bytes("solve", 0, n, iters, cells, "mg")
    per_cell = 16 + 28 + 12 + 12 * (4 * bench.MG_SWEEPS - 1) + 0.5 + 5 * (4 * bench.MG_SWEEPS + 2)
    assert bench.MG_SWEEPS != 2 or per_cell == 190.5
    assert mg == int(21 * C + iters * (per_cell * cells +
                                       15 * (4 * bench.MG_SWEEPS + 2) * bench.mg_coarse_cells(n)))


def test_kernel_bytes():
    n, P, cells = 128, 1000, 657280
    C = n ** 3
    # the solve kernel: its iterations only (the refinement's setup pass is
    # in other kernels)
    mg1 = bench.stage_bytes("solve", 0, n, 1, cells, "mg") - 21 * C
    assert bench.kernel_bytes("k_cg_mg", P, n, 2, 17, cells, "mg") == mg1 * 17
    # a gather: its stage's bytes once per step
    assert bench.kernel_bytes("k_density", P, n, 2, 17) == 2 * bench.stage_bytes("density", P, n, 0)
    # the corrector's two kernels
    assert bench.kernel_bytes("k_spring_inline", P, n, 1, 0) == 32 * P + 4 * C
    assert bench.kernel_bytes("k_resample_inline", P, n, 1, 0) == 60 * P + 4 * C
    assert bench.kernel_bytes("k_unknown", P, n, 1, 0) == 0


def test_roofline_note():
    assert bench.roofline_note("k_cg_mg", None, 10) is None
    assert "stays in L2" in bench.roofline_note("k_cg_mg", 39_000_000, 2_000_000_000)
    assert "stays in L2" not in bench.roofline_note("k_cg_mg", 1_900_000_000, 2_000_000_000)
    assert "L1 data pipe" in bench.roofline_note("k_spring_inline", None, 10)


def test_traffic_scales_with_particles(tmp_path, monkeypatch):
    f = tmp_path / "traffic.txt"
    f.write_text("# kernel n bytes particles\nk_density 128 1000 100\n")
    monkeypatch.setattr(bench, "TRAFFIC", str(f))
    assert bench.measured_traffic("k_density", 128, 100) == (1000, "measured")
    t, src = bench.measured_traffic("k_density", 256, 400)
    assert t == 4000 and "scaled" in src
    assert bench.measured_traffic("k_p2g_cells", 256, 400) == (None, None)


def test_committed_traffic_rows_name_profiled_kernels():
    """Every row of profiles/traffic.txt names a kernel that the per-kernel
    profile reports, so the bench can find it."""
    kernels = {"k_density", "k_p2g_cells", "k_spring_inline", "k_resample_inline",
               "k_flip_advect", "k_cg_mg", "k_cg_cg1", "k_cg_ic", "k_cg"}
    with open(bench.TRAFFIC) as f:
        rows = [ln.split() for ln in f if ln.strip() and not ln.startswith("#")]
    assert rows and all(len(r) == 4 and r[0] in kernels for r in rows)

"""Benchmark of the FLIP step on GB300.

One step = one simulateStep of the hot path (sort, density, P2G, markWater,
projection with PCG refined to a true relative residual of 1e-6, G2P + FLIP
blend, advection with wall constraint and reposition, position correction)
on the sphere-into-pool scene at N=256 (pool depth 0.25, sphere r 0.15 at
(0.5,0.75,0.5) falling at 2 m/s; 8 particles per liquid cell, about 34.8M
particles), synthetic seeded data. --scene dam_break --n 128 runs the N=128
dam break (column x<0.4, y<0.8; 5.2M particles).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line. `value` is particle-steps/s over all ranks with the
state resident on the device; `e2e` is the same metric through the C ABI with
the particle state copied from pinned host memory before each step and back
after it. Multi-GPU runs are independent replicas (the step has no exchange).
The CPU baseline (and the reference arm) time the CPU restatement of the
reference step on the host cores: the reference arm on the benchmark's own
workload under a time cap (it reports the steps it actually ran), the
CPU-baseline leg of the GPU arm on a bounded sample (the same scene at a
quarter of the grid size, a warm-up step and three timed steps).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "learned-warm-start vs plain MIC-PCG ms/solve @ rel-res 1e-6; particle-steps/s"
UNIT = "particle-steps/s"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC = os.path.join(ROOT, "profiles", "traffic.txt")
FALLBACK_HBM = 6800.0


WEIGHTS = os.path.join(ROOT, "flip3d_gb300", "unet_weights.bin")


def run_batch(args):
    """Aggregate particle-steps/s of many small scenes stepped together
    (one CUDA graph per scene, every scene on its own stream, no host waits
    between scenes) against the same scenes stepped one at a time."""
    # the members' streams get hardware work queues of their own (the
    # default 8 queues make streams that share one wait for each other);
    # read when the CUDA context is created
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    import torch

    from flip3d_gb300 import gpu, scenes
    gpu.load()
    torch.cuda.set_device(0)
    scs = [scenes.batch_scene(1000 + i) for i in range(args.batch_scenes)]
    sims = []
    for i, sc in enumerate(scs):
        mg = args.precond == "mg" and sc.n % 4 == 0 and sc.n >= 8
        s = gpu.Simulation(gpu.default_params(sc.n, sc.count, rel_tol=1e-6, seed=i,
                                              solve_mode=gpu.SOLVE_FAST,
                                              precond=gpu.PRECOND_MG if mg else gpu.PRECOND_JACOBI,
                                              mg_sweeps=MG_SWEEPS,
                                              arith=gpu.ARITH_FAST if args.arith == "fast"
                                              else gpu.ARITH_REF))
        s.set_scene(sc)
        s.calibrate_max_density()
        sims.append(s)
    P = sum(sc.count for sc in scs)
    # one at a time: each scene's step completes before the next starts
    for _ in range(args.warmup):
        for s in sims:
            s.step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for s in sims:
            s.step()
            s.sync()
    t_seq = time.perf_counter() - t0
    # together, the solves' share of the GPU tuned on the systems of one step
    b = gpu.Batch(sims)
    b.capture()
    b.step()
    b.sync()
    share = b.tune()
    tuning = [ln for ln in gpu.autotune_report().splitlines() if ln.startswith("batch solve share")]
    clocks = ClockSampler(0)
    clocks.start()
    clocks.wait_first()
    for _ in range(args.warmup):
        b.step()
    b.sync()
    launches0 = sum(s.launches for s in sims)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        b.step()
    b.sync()
    t1 = time.perf_counter()
    t_bat = t1 - t0
    clk = clocks.stop((t0, t1))
    launches = sum(s.launches for s in sims) - launches0
    value = P * args.steps / t_bat
    sizes = {}
    for sc in scs:
        sizes[sc.n] = sizes.get(sc.n, 0) + 1
    print(json.dumps({
        "metric": "particle-steps/s, batched uneven scenes", "value": value, "unit": UNIT,
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_bat / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{len(scs)} scenes, N uniform from {{24,32,48,64,96}} "
                               f"({sizes}), pool U(0.1,0.4) + sphere r U(0.08,0.2), "
                               f"{P} particles in all",
                   "solver": f"FP32 PCG {args.precond}, double-float dots, refined to a true "
                             f"relative residual of 1e-6",
                   "arith": f"particle gathers {args.arith}",
                   "queues": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
                   "timing": "host wall clock around device-synchronised steps",
                   "l2": "inputs larger than L2"},
        "one_at_a_time": {"value": P * args.steps / t_seq, "ms_per_step": t_seq / args.steps * 1e3},
        "speedup_vs_one_at_a_time": t_seq / t_bat,
        "solve_share": {"share": share, "grids": [s.solve_blocks() for s in sims],
                        "tuning": tuning[-1] if tuning else None},
        "gpu_launches": launches, "clocks": clk}))


def solver_comparison(gpu, sim, prm, n, systems=3):
    """ms per solve, CG iterations and the FP64 true relative residual on
    pressure systems captured from the next steps of the run, each solved
    from the same previous-step guess (the reference's own warm start) to a
    true relative residual of 1e-6 by: plain Jacobi, MIC(0) and multigrid
    PCG, and each of them again with the learned warm start (trained
    weights in flip3d_gb300/). The network's contribution is the ratio on
    the same preconditioner (learned_X_vs_plain_X); the ratio against plain
    MIC(0) of the fastest learned variant also counts the change of
    preconditioner and is labelled so."""
    sim.set_capture(True)
    caught = []
    for _ in range(systems):
        sim.step()
        caught.append(sim.solve_system())
    sim.set_capture(False)
    net = None
    if os.path.exists(WEIGHTS) and n % 8 == 0:
        net = gpu.UNet(seed=0)
        net.load(WEIGHTS)
    pres = [("jacobi", gpu.PRECOND_JACOBI, 0.0), ("mic", gpu.PRECOND_IC, 0.97)]
    if n % 4 == 0:
        pres.append(("mg", gpu.PRECOND_MG, 0.0))
    variants = [(f"plain_{k}", pre, tau, None) for k, pre, tau in pres]
    if net is not None:
        variants += [(f"learned_{k}", pre, tau, net) for k, pre, tau in pres]
    out = {}
    for name, pre, tau, w in variants:
        p = gpu.Params.from_buffer_copy(prm)
        p.precond, p.mic_tau, p.solve_mode = pre, tau, gpu.SOLVE_FAST
        sim.set_params(p)
        sim.set_warm_start(w)
        ms, it, wms, passes, rel, guess = [], [], [], [], [], []
        for A, L, b, x0, _, _ in caught:
            for rep in range(2):  # the first solve of a variant warms it up
                sim.set_grid(A=A, L=L, press=x0, div=-b)
                st = sim.solve()
            ms.append(st.ms)
            it.append(st.iterations)
            wms.append(st.warm_ms)
            passes.append(st.refine_passes)
            rel.append((st.r2_true / st.b2) ** 0.5 if st.b2 > 0 else 0.0)
            if w is not None and st.r2_prev > 0:
                guess.append((st.r2_guess / st.r2_prev) ** 0.5)
        out[name] = {"ms_per_solve": statistics.mean(ms), "iters": statistics.mean(it),
                     "refine_passes": statistics.mean(passes),
                     "true_rel_residual_fp64": max(rel)}
        if w is not None:
            out[name]["warm_start_ms"] = statistics.mean(wms)
            if guess:
                out[name]["guess_residual_vs_previous_step"] = statistics.mean(guess)
    sim.set_warm_start(None)
    sim.set_params(prm)
    for k, _, _ in pres:
        if f"learned_{k}" in out:
            a, b = out[f"learned_{k}"], out[f"plain_{k}"]
            out[f"learned_{k}_vs_plain_{k}"] = {"ms": a["ms_per_solve"] / b["ms_per_solve"],
                                                "iters": a["iters"] / max(b["iters"], 1e-9)}
    if "plain_mg" in out:
        out["plain_mg_vs_plain_mic"] = out["plain_mg"]["ms_per_solve"] / \
            out["plain_mic"]["ms_per_solve"]
    learned = [k for k in out if k.startswith("learned_") and "_vs_" not in k]
    if learned:
        best = min(learned, key=lambda k: out[k]["ms_per_solve"])
        out["fastest_learned_vs_plain_mic"] = {
            "variant": best,
            "ms": out[best]["ms_per_solve"] / out["plain_mic"]["ms_per_solve"],
            "note": "includes the change of preconditioner; the network's own effect is "
                    "learned_X_vs_plain_X"}
    out["systems"] = systems
    out["start"] = "previous-step pressure (the reference's warm start, src/flip3D.cpp:49,659)"
    return out


def measured_traffic(kernel, n, particles):
    """DRAM bytes of the kernel per step (per solve for a solve kernel; its
    dram__bytes_read.sum + dram__bytes_write.sum) from the ncu summaries in
    profiles/, and how it was obtained: measured at this grid size, or
    scaled from a capture of a smaller workload by the particle count (the
    gathers' traffic grows with the particles they touch). (None, None)
    when the kernel was not captured."""
    rows = []
    try:
        with open(TRAFFIC) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 4 and not line.startswith("#") and parts[0] == kernel:
                    rows.append((int(parts[1]), int(parts[2]), int(parts[3])))
    except OSError:
        pass
    for rn, rb, rp in rows:
        if rn == n:
            return rb, "measured"
    if rows:
        rn, rb, rp = max(rows)
        return int(rb * particles / rp), f"scaled from N={rn} ({rp} particles) by particle count"
    return None, None


GATHER_KERNELS = ("k_density", "k_p2g_cells", "k_spring_inline", "k_resample_inline")
PROFILED_STEPS = 2


def kernel_bytes(kernel, P, n, steps, iters, sweep_cells=None, precond="jacobi"):
    """Algorithmic bytes of all launches of one of the profiled kernels over
    `steps` steps whose solves took `iters` iterations in all, by the model
    of stage_bytes(): the persistent solve kernel its iterations (the
    refinement's residual and update kernels are not part of it), each
    gather one call of its stage; the corrector's two kernels split its
    bytes: the spring reads the sorted positions and the permutation and
    writes positions (32 B per particle), the resample reads the sorted
    positions and velocities, the moved position and the permutation and
    writes velocities (60 B); both read the cell starts."""
    C = n ** 3
    if kernel.startswith("k_cg"):
        per = stage_bytes("solve", P, n, 1, sweep_cells, precond) - 21 * C
        return per * iters
    per_step = {
        "k_density": stage_bytes("density", P, n, 0),
        "k_p2g_cells": stage_bytes("p2g", P, n, 0),
        "k_spring_inline": P * 32 + 4 * C,
        "k_resample_inline": P * 60 + 4 * C,
        "k_flip_advect": stage_bytes("g2p_flip", P, n, 0),
    }.get(kernel, 0)
    return per_step * steps


def roofline_note(kernel, traffic, nbytes):
    """Reading of the roofline fraction against the kernel's DRAM traffic."""
    notes = []
    if kernel in GATHER_KERNELS:
        notes.append("a particle gather: bound by the L1 data pipe (one 16-byte neighbour "
                     "load per particle pair, 85-91 % of its peak in ncu), not by HBM")
    if traffic is not None and nbytes:
        if traffic < 0.2 * nbytes:
            notes.append(f"ncu DRAM traffic {traffic} B per call against {nbytes} algorithmic "
                         "B: the working set stays in L2 (grid barriers and L2 latency bound "
                         "it)")
        else:
            notes.append(f"ncu DRAM traffic {traffic} B per call against {nbytes} "
                         "algorithmic B")
    return "; ".join(notes) if notes else None


def hbm_peak():
    try:
        with open(PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


def liquid_chunk_cells(A):
    """Cells of the 128-cell chunks (32 quads of the x-major order) that hold
    liquid: the cells the single-reduction PCG sweeps every iteration."""
    import numpy as np

    f = np.asarray(A).reshape(-1) == 1
    pad = (-f.size) % 128
    if pad:
        f = np.concatenate([f, np.zeros(pad, dtype=bool)])
    return int(f.reshape(-1, 128).any(axis=1).sum()) * 128


MG_SWEEPS = 2  # red-black sweeps per level and side of the V-cycle (the library default)


def mg_coarse_cells(n):
    """Cells of the multigrid levels below the solver's grid (ceil(m/2) per
    axis down to at most 4)."""
    tot, m = 0, n
    while m > 4:
        m = (m + 1) // 2
        tot += m ** 3
    return tot


def stage_bytes(stage, P, n, iters, sweep_cells=None, precond="jacobi"):
    """Algorithmic bytes of one call of a stage: every input read once and
    every output written once, nothing else. The PCG solve is one setup pass
    over the grid (A, x, b, M^-1 read, 13 B; r and x written, 8 B) and per
    iteration, over the cells of the liquid chunks (sweep_cells; the whole
    grid when not given):
      Jacobi (single reduction): 49 B: A 1 + diagonal 4 + M^-1 4 + U, Wt, St,
        p, x 4 each read, U, Wt, St, p, x 4 each written;
      multigrid with nu smoothing sweeps: on the solver's grid p' = z + beta p
        and A p' 16 B, the x/r update with the first half sweep 28 B, the
        residual 12 B, 4 nu - 1 more half sweeps 12 B each (the one after the
        coarse correction also reads the parents, 0.5 B), and every one of
        those 4 nu + 2 passes reads A and the diagonal, 5 B (nu = 2: 190.5 B);
        plus 15 B per pass on every coarser level, 4 nu + 2 passes (half
        sweeps, residual, the restriction's writes, prolongation)."""
    C = n ** 3
    F = 3 * (n + 1) * n * n
    cells = C if sweep_cells is None else sweep_cells
    if precond == "mg":
        hs = 4 * MG_SWEEPS - 1
        per_cell = 16 + 28 + 12 + 12 * hs + 0.5 + 5 * (hs + 3)
        solve_iter = per_cell * cells + 15 * (4 * MG_SWEEPS + 2) * mg_coarse_cells(n)
    else:
        solve_iter = 49 * cells
    table = {
        # count: pos 12 r, key 4 w, rank 4 w; scatter: key+rank 8 r, perm 4 w;
        # cell counts/starts 3*4*C; payload: perm 4 + pos 12 + vel 12 + type 1 + dens 4 r,
        # 52 w (spos, spg, svel 16 each, sdens 4)
        "sort": P * (12 + 8 + 8 + 4) + 12 * C + P * (33 + 52),
        "density": P * (16 + 4) + 4 * C,
        "mark_water": P * 8 + 4 * C + 5 * C,
        "p2g": P * 32 + 4 * C + C + 2 * 4 * F,
        "divergence": C + 4 * F + 4 * C,
        "solve": int(21 * C + max(iters, 1) * solve_iter),
        "gradient": 4 * F * 2 + 9 * C,
        "extrapolate": 4 * F * 3 + C,
        # FLIP blend fused with advect_particle: pos, vel, type, dens read;
        # pos, vel, stuck flag written; the new grid and its change read once
        "g2p_flip": P * (12 + 12 + 1 + 4 + 12 + 12 + 1) + 2 * 4 * F + C,
        "advect": 0,
        "reposition": P * 1 + C,
        "correct": P * (16 + 16 + 12 + 12 + 4) + 4 * C,
    }
    return table.get(stage, 0)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms. Started
    before the warm-up (its first sample is awaited, so the tool's start-up
    stays out of the timed region); stop(window) keeps the samples that
    arrived during the timed window, or the two nearest to it when the
    window is shorter than the sampling period."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows = []
        self.proc = None
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.perf_counter(), [x.strip() for x in line.split(",")]))

    def wait_first(self, timeout=5.0):
        t0 = time.perf_counter()
        while self.proc and not self.rows and time.perf_counter() - t0 < timeout:
            time.sleep(0.01)

    def stop(self, window=None):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        rows = self.rows
        if window is not None and rows:
            a, b = window
            inside = [r for r in rows if a <= r[0] <= b + 0.25]
            rows = inside if inside else sorted(
                rows, key=lambda r: min(abs(r[0] - a), abs(r[0] - b)))[:2]
        rows = [r[1] for r in rows]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for i, nm in enumerate(names):
                    if r[5 + i].lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_step_rate(scene, warmup=1, steps=3):
    """Time the CPU restatement of the reference step (all host threads):
    warm-up steps, then `steps` timed steps."""
    from oracle import pyoracle as orc
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    prm = orc.params(scene.n, orc.PRECOND_REF, rel_tol=1e-6, seed=1)
    sim = orc.Sim(scene, prm, orc.max_density(scene.n))
    for _ in range(warmup):
        sim.step()
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.step()
    dt = time.perf_counter() - t0
    return scene.count * steps / dt, cores, steps, dt


def max_over_ranks(value, world, device):
    """The largest value over the ranks of the current process group (the
    slowest replica's time); the value itself with one rank."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(particles_per_rank, world, steps, seconds):
    """Whole-job particle-steps/s of `world` replicas that each advanced
    `particles_per_rank` particles `steps` times in at most `seconds`."""
    return particles_per_rank * world * steps / seconds


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


REF_WARMUP_CAP_S = 60.0   # warm-up steps stop once this much time has passed
REF_TIMED_CAP_S = 150.0   # timed steps stop once this much time has passed (>= 1 step)


def run_reference(args):
    """The reference's step on the host cores (the CPU restatement, pinned
    bit-exact to the reference's own build) on the benchmark's workload.
    At N=256 one step takes minutes, so warm-up and timed steps run under
    time caps; the line reports the steps actually run."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from flip3d_gb300 import scenes
    from oracle import pyoracle as orc
    sc = getattr(scenes, args.scene)(args.n, seed=0)
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    prm = orc.params(sc.n, orc.PRECOND_REF, rel_tol=1e-6, seed=1)
    sim = orc.Sim(sc, prm, orc.max_density(sc.n))
    t0 = time.perf_counter()
    warm = 0
    while warm < args.warmup and (warm == 0 or time.perf_counter() - t0 < REF_WARMUP_CAP_S):
        sim.step()
        warm += 1
    t0 = time.perf_counter()
    steps = 0
    while steps < args.steps and (steps == 0 or time.perf_counter() - t0 < REF_TIMED_CAP_S):
        sim.step()
        steps += 1
    dt = time.perf_counter() - t0
    value = sc.count * steps / dt
    capped = steps < args.steps or warm < args.warmup
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
           "n_gpus": args.gpus, "steps": steps, "warmup": warm,
           "requested": {"steps": args.steps, "warmup": args.warmup},
           "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"{args.scene} N={args.n}, 8 particles/cell, rel-res 1e-6 "
                                  f"({sc.count} particles)",
                      "particles": sc.count, "grid": args.n,
                      "solver": "the reference's PCG (its preconditioner, FP32 x), relative "
                                "tolerance 1e-6 on its recursive residual",
                      "time_caps_s": {"warmup": REF_WARMUP_CAP_S, "timed": REF_TIMED_CAP_S},
                      "capped": capped,
                      "note": "the reference's own method: the GPU arm solves with multigrid "
                              "PCG refined to a true relative residual of 1e-6 and FAST "
                              "gathers, so a ratio of the two arms includes that change of "
                              "method"},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                            "sample": f"{warm} warm-up + {steps} timed full steps of "
                                      f"{args.scene} N={args.n} ({sc.count} particles), "
                                      f"{dt:.1f} s timed"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--precond", default="mg", choices=["jacobi", "ic", "mic", "mg", "ref"],
                    help="preconditioner of the FAST-mode PCG (mg: multigrid V-cycle)")
    ap.add_argument("--arith", default="fast", choices=["fast", "ref"],
                    help="particle-gather arithmetic: native FP32 (fast) or the reference's "
                         "float expressions bit for bit (ref)")
    ap.add_argument("--scene", default="sphere_into_pool",
                    choices=["dam_break", "sphere_into_pool"],
                    help="dam_break (column x<0.4, y<0.8) or sphere_into_pool (pool 0.25, "
                         "sphere r 0.15 falling at 2 m/s)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-solver-comparison", action="store_true",
                    help="skip the plain/MIC/learned solver comparison (profiling runs)")
    ap.add_argument("--batch-scenes", type=int, default=0,
                    help="run the batched workload instead: this many independent scenes "
                         "with N uniform from {24,32,48,64,96}, stepped together (captured "
                         "CUDA graphs on per-scene streams) and one at a time")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.precond == "mg" and (args.n % 4 != 0 or args.n < 8):
        args.precond = "jacobi"  # the multigrid solver works on quads of cells
    if args.batch_scenes > 0:
        run_batch(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return

    import numpy as np
    import torch

    from flip3d_gb300 import gpu, scenes

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    t_build = time.perf_counter()
    sc = getattr(scenes, args.scene)(args.n, seed=rank)
    t_build = time.perf_counter() - t_build
    P = sc.count
    pre = {"jacobi": gpu.PRECOND_JACOBI, "ic": gpu.PRECOND_IC, "mic": gpu.PRECOND_IC,
           "mg": gpu.PRECOND_MG, "ref": gpu.PRECOND_REF}[args.precond]
    mode = gpu.SOLVE_REF if args.precond == "ref" else gpu.SOLVE_FAST
    prm = gpu.default_params(args.n, P, rel_tol=1e-6, solve_mode=mode, precond=pre, seed=1,
                             mic_tau=0.97 if args.precond == "mic" else 0.0, mg_sweeps=MG_SWEEPS,
                             arith=gpu.ARITH_FAST if args.arith == "fast" else gpu.ARITH_REF)
    sim = gpu.Simulation(prm)
    t_up = time.perf_counter()
    sim.set_scene(sc)
    t_up = time.perf_counter() - t_up
    # the same particles seeded on the device (flipgpu_seed_scene)
    t_seed = time.perf_counter()
    sim.seed_scene(sc.objects, seed=rank)
    t_seed = time.perf_counter() - t_seed
    setup = {"host_build_s": round(t_build, 4), "host_upload_s": round(t_up, 4),
             "device_seed_s": round(t_seed, 4),
             "note": "scene setup, not part of value: numpy build + upload vs flipgpu_seed_scene"}
    sim.calibrate_max_density()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # the library launches on this stream; the events are recorded on it
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    solve_ms, iters, true_rel, passes = [], [], [], []
    clocks = ClockSampler(local)
    clocks.start()
    clocks.wait_first()
    # the end-to-end loop below restarts from the state before the last
    # warm-up steps, so that both timed loops run the same steps of the
    # simulation (later steps, after the sphere has reached the pool, cost
    # more)
    e2e_warm = min(2, args.warmup)
    for _ in range(args.warmup - e2e_warm):
        sim.step()
    sim.sync()
    snap_step = args.warmup - e2e_warm
    snap_pos, snap_vel, _, _ = sim.get_particles()
    snap_press = sim.get_grid()[3]
    sim.set_step(snap_step)
    for _ in range(e2e_warm):
        sim.step()
    barrier()
    launches0 = sim.launches
    start_ev = torch.cuda.Event(enable_timing=True)
    end_ev = torch.cuda.Event(enable_timing=True)
    stream.synchronize()
    t_clk0 = time.perf_counter()
    start_ev.record(stream)
    for _ in range(args.steps):
        st = sim.step()
        solve_ms.append(st.ms)
        iters.append(st.iterations)
        passes.append(st.refine_passes)
        if st.b2 > 0:
            true_rel.append((st.r2_true / st.b2) ** 0.5)
    end_ev.record(stream)
    stream.synchronize()
    t_clk1 = time.perf_counter()
    barrier()
    clk = clocks.stop((t_clk0, t_clk1))
    launches = sim.launches - launches0
    ms = start_ev.elapsed_time(end_ev)
    ms = max_over_ranks(ms, world, "cuda")
    value = replica_throughput(P, world, args.steps, ms / 1e3)

    # per-stage and per-kernel profile (a separate pass: CUDA events between
    # the stages and around each launch of the main kernels)
    sim.set_profiling(True)
    prof_iters = []
    for _ in range(PROFILED_STEPS):
        st = sim.step()
        prof_iters.append(int(st.iterations))
    prof = sim.profile()
    kprof = sim.kernel_profile()
    sim.set_profiling(False)
    sweep_cells = liquid_chunk_cells(sim.get_grid()[1])
    # the roofline's kernel: the one with the most device time
    dom = max(kprof, key=lambda k: kprof[k][0])
    k_ms, k_calls = kprof[dom]
    dom_ms = k_ms / max(k_calls, 1)
    nbytes = kernel_bytes(dom, P, args.n, PROFILED_STEPS, sum(prof_iters), sweep_cells,
                          args.precond) / max(k_calls, 1)
    peak, peak_kind = hbm_peak()
    achieved = nbytes / (dom_ms / 1e3) / 1e9
    traffic, traffic_src = measured_traffic(dom, args.n, P)
    if traffic is not None:
        # a row is per step (per solve for a solve kernel): per launch here
        traffic = int(traffic * PROFILED_STEPS / max(k_calls, 1))

    # end to end through the C ABI with pinned host buffers: every step
    # uploads the particle state, steps and downloads it (flipgpu_step_host,
    # which overlaps the transfers with the step)
    hpos = torch.empty((P, 3), dtype=torch.float32, pin_memory=True)
    hvel = torch.empty((P, 3), dtype=torch.float32, pin_memory=True)
    hp, hv = hpos.numpy(), hvel.numpy()
    hp[:] = snap_pos
    hv[:] = snap_vel
    sim.put_state(snap_pos, snap_vel)
    sim.set_grid(press=snap_press)
    sim.set_step(snap_step)
    for _ in range(e2e_warm):
        sim.step_host(hp, hv, hp, hv)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sim.step_host(hp, hv, hp, hv)
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, world, "cuda")
    e2e = replica_throughput(P, world, args.steps, e2e_s)

    # the metric's solver comparison on systems of this run (not in `value`)
    solve_cmp = None if args.no_solver_comparison else solver_comparison(gpu, sim, prm, args.n)

    # mesher::generateMesh on the last step's lists (device only, not in `value`)
    sim.mesh_counts()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mesh_v, mesh_f = sim.mesh_counts()
    mesh_ms = (time.perf_counter() - t0) * 1e3

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # a bounded sample: the same scene at a quarter of the grid size (a
        # step of the full workload takes minutes on the host cores; the
        # reference arm times that one under a time cap)
        ns = max(16, (args.n // 4) // 4 * 4)
        sample = getattr(scenes, args.scene)(ns, seed=0)
        rate, cores, steps, dt = cpu_step_rate(sample, warmup=1, steps=3)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"1 warm-up + {steps} timed full steps of {args.scene} N={ns} "
                         f"({sample.count} particles), {dt:.1f} s timed; the reference arm "
                         f"(--impl reference) times N={args.n} itself"}

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"{args.scene} N={args.n}, 8 particles/cell, rel-res 1e-6",
                       "particles": P, "grid": args.n,
                       "solver": f"FP32 PCG {args.precond}" +
                                 (f" ({MG_SWEEPS} red-black sweeps per level)"
                                  if args.precond == "mg" else "") +
                                 ", double-float dots, mixed-precision iterative refinement "
                                 "(double-float iterate) to a true relative residual of 1e-6",
                       "arith": f"particle gathers {args.arith} "
                                f"({'native FP32' if args.arith == 'fast' else 'reference bit-exact'})",
                       "l2": "inputs larger than L2 (particle state alone "
                             f"{P * 28 / 1e9:.2f} GB)",
                       "parallelism": f"replicas x{world}"},
            "solve": {"ms_per_solve": statistics.mean(solve_ms), "iters": statistics.mean(iters),
                      "refine_passes": statistics.mean(passes),
                      "kind": f"refined PCG ({args.precond}), previous-step start",
                      "true_rel_residual_fp64": max(true_rel) if true_rel else None},
            "solver_comparison": solve_cmp,
            "setup": setup,
            "stages_ms": {k: round(v[0] / max(v[1], 1), 4) for k, v in prof.items()},
            "mesh": {"ms": mesh_ms, "vertices": mesh_v, "faces": mesh_f,
                     "note": "mesher::generateMesh after the last step, host-timed, "
                             "not part of value"},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "peak_source": peak_kind, "algorithmic_bytes": nbytes,
                         "ms_per_launch": dom_ms,
                         "launches_per_step": k_calls / PROFILED_STEPS,
                         "timing": "CUDA events around each launch on the handle's stream, "
                                   f"{PROFILED_STEPS} profiled steps after the timed ones",
                         "bytes_model": "kernel_bytes(): every input read once, every output "
                                        "written once, per launch; a solve kernel counts its "
                                        "solver-grid passes over the liquid chunks only",
                         "kernels_ms_per_step": {k: round(v[0] / PROFILED_STEPS, 4)
                                                 for k, v in sorted(kprof.items(),
                                                                    key=lambda t: -t[1][0])},
                         "sweep_cells": sweep_cells, "traffic_source": traffic_src,
                         "note": roofline_note(dom, traffic, nbytes)},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": P * 24,
                    "d2h_bytes_per_step": P * 24,
                    "steps": "the same steps as value: restarted from the particles, "
                             "pressure and step counter saved before the last "
                             f"{e2e_warm} warm-up steps"},
            "gpu_launches": launches,
            "clocks": clk,
        }
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

"""Training data, training loop and evaluation of the learned warm start.

The network (libflipgpu's flipunet_* calls: forward, backward and Adam are
the library's own CUDA kernels) learns, from systems the plain FAST solver
solved on seeded random scenes (1-4 liquid boxes/spheres, pool depth
U(0, 0.4), velocities N(0, 1)), the correction from the previous step's
pressure to the solution. Torch holds the device tensors; it is plumbing.

    python -m flip3d_gb300.train_unet --n 128 --coarsen 2 --scenes 40 --steps 50 \\
        --every 5 --epochs 30 --out flip3d_gb300/unet_weights.bin
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import gpu, scenes

KEYS = ("A", "L", "b", "x0", "r0", "x")


def solver_params(n, count, seed=0):
    return gpu.default_params(n, max(count, 1), rel_tol=1e-6, solve_mode=gpu.SOLVE_FAST,
                              precond=gpu.PRECOND_JACOBI, seed=seed)


def collect(n, seeds, steps, every, device="cuda", keys=KEYS):
    """(A, L, b, x0, r0, x) of every `every`-th solve of each seeded scene
    (those of `keys`), as device tensors [systems, n^3] written in place into
    tensors allocated once (20,000 systems at n = 64 hold about 90 GB
    without L)."""
    import torch
    seeds = list(seeds)
    count = len(seeds) * (steps // every)
    out = {k: torch.empty((count, n ** 3), dtype=torch.uint8 if k == "A" else torch.float32,
                          device=device) for k in keys}
    m = 0
    for seed in seeds:
        sc = scenes.random_scene(n, int(seed))
        sim = gpu.Simulation(solver_params(n, sc.count, int(seed)))
        sim.set_scene(sc)
        sim.calibrate_max_density()
        sim.set_capture(True)
        for k in range(1, steps + 1):
            sim.step()
            if k % every:
                continue
            dst = [out[key][m] if key in out else None for key in KEYS]
            sim.solve_system(dev=[None if x is None else x.data_ptr() for x in dst])
            sim.sync()
            m += 1
        sim.close()
    return out


def train(net, data, n, epochs, batch=16, lr=1e-3, seed=0, log=None, lr_end=None):
    """Adam over shuffled mini-batches with the learning rate decaying
    (cosine) from lr to lr_end (lr/20 by default); returns the mean loss per
    epoch."""
    import torch
    count = data["A"].shape[0]
    batch = min(batch, count)
    g = torch.Generator().manual_seed(seed)
    history = []
    lr_end = lr / 20.0 if lr_end is None else lr_end
    per_epoch = max(1, count // batch)
    total = epochs * per_epoch
    it = 0
    for ep in range(epochs):
        order = torch.randperm(count, generator=g)
        losses = []
        for i in range(0, count - batch + 1, batch):
            rate = lr_end + 0.5 * (lr - lr_end) * (1.0 + np.cos(np.pi * it / max(total - 1, 1)))
            it += 1
            idx = order[i:i + batch].to(data["A"].device)
            A, b, x0, r0, x = (data[k].index_select(0, idx).contiguous()
                               for k in ("A", "b", "x0", "r0", "x"))
            torch.cuda.synchronize()
            losses.append(net.train_step(n, batch, A.data_ptr(), b.data_ptr(), x0.data_ptr(),
                                         r0.data_ptr(), x.data_ptr(), float(rate)))
        history.append(float(np.mean(losses)))
        if log:
            log(f"epoch {ep + 1}/{epochs}: loss {history[-1]:.4g}")
    return history


def prediction_error(net, data, n):
    """Median over systems of ||d - (x - x0)|| / ||x - x0|| on the liquid,
    with d the network's correction scaled by its least-squares factor."""
    import torch
    errs = []
    for i in range(data["A"].shape[0]):
        A, b, x0, r0, x = (data[k][i:i + 1].contiguous() for k in ("A", "b", "x0", "r0", "x"))
        d = torch.zeros_like(b)
        torch.cuda.synchronize()
        net.predict(n, 1, A.data_ptr(), b.data_ptr(), x0.data_ptr(), r0.data_ptr(), d.data_ptr())
        torch.cuda.synchronize()
        fl = A == 1
        want = (x - x0)[fl].double()
        got = d[fl].double()
        den = float(want.norm())
        if den == 0.0:
            continue
        c = float((got * want).sum() / max(float((got * got).sum()), 1e-300))
        errs.append(float((c * got - want).norm()) / den)
    return float(np.median(errs)) if errs else 0.0


PRECONDS = {"jacobi": (gpu.PRECOND_JACOBI, 0.0), "mic": (gpu.PRECOND_IC, 0.97),
            "mg": (gpu.PRECOND_MG, 0.0)}


def evaluate(net, data, n, precond="jacobi"):
    """Each held-out system solved from its previous-step guess and from the
    learned warm start with the same preconditioner (refined to a true
    relative residual of 1e-6): CG iterations and device ms per solve."""
    prm = solver_params(n, 1)
    prm.precond, prm.mic_tau = PRECONDS[precond]
    sim = gpu.Simulation(prm)
    plain, learned = [], []
    for i in range(data["A"].shape[0]):
        A, L, b, x0 = (data[k][i].cpu().numpy() for k in ("A", "L", "b", "x0"))
        sim.set_warm_start(None)
        sim.set_grid(A=A, L=L, press=x0, div=-b)
        st = sim.solve()
        plain.append((st.iterations, st.ms))
        sim.set_warm_start(net)
        sim.set_grid(A=A, L=L, press=x0, div=-b)
        st = sim.solve()
        learned.append((st.iterations, st.ms, st.r2_prev, st.r2_guess, st.warm_ms))
    sim.set_warm_start(None)
    p, q = np.array(plain), np.array(learned)
    return {"systems": int(len(plain)), "plain_iters": float(p[:, 0].mean()),
            "plain_ms": float(p[:, 1].mean()), "learned_iters": float(q[:, 0].mean()),
            "learned_ms": float(q[:, 1].mean()), "warm_ms": float(q[:, 4].mean()),
            "residual_ratio": float(np.median(np.sqrt(q[:, 3] / np.maximum(q[:, 2], 1e-300)))),
            "pred_rel_err": prediction_error(net, data, n)}


def time_predict(n, weights=None, reps=10, tcgen05=True):
    """Device ms of one forward pass (flipunet_predict) on a seeded random
    n^3 system with 70 % liquid, after two warm-up calls."""
    import torch
    rng = np.random.default_rng(5)
    A = torch.tensor((rng.random(n ** 3) < 0.7).astype(np.uint8), device="cuda")
    b, x0, r0 = (torch.tensor(rng.normal(0, 1, n ** 3).astype(np.float32), device="cuda")
                 for _ in range(3))
    net = gpu.UNet(seed=4)
    if weights:
        net.load(weights)
    net.set_tensor_path(tcgen05)
    d = torch.zeros(n ** 3, dtype=torch.float32, device="cuda")
    args = [t.data_ptr() for t in (A, b, x0, r0, d)]
    for _ in range(2):
        net.predict(n, 1, *args)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        net.predict(n, 1, *args)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--scenes", type=int, default=40)
    ap.add_argument("--holdout", type=int, default=4)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--every", type=int, default=5)
    ap.add_argument("--epochs", type=int, default=4)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--coarsen", type=int, default=0,
                    help="run the network on the grid pooled this many times")
    ap.add_argument("--init", default=None, help="start from these weights")
    ap.add_argument("--time-predict", type=int, default=0, metavar="N",
                    help="only time the forward pass on an N^3 system (both tensor paths)")
    ap.add_argument("--out", default=None)
    ap.add_argument("--eval-precond", default="jacobi",
                    help="comma-separated preconditioners of the held-out evaluation "
                         "(jacobi, mic, mg)")
    ap.add_argument("--eval-steps", default="minres",
                    help="comma-separated step rules along the network's correction to "
                         "evaluate: minres (least residual, the library's default) and/or "
                         "anorm (least A-norm error); set through FLIPGPU_WARM_STEP")
    ap.add_argument("--eval-n", default="",
                    help="comma-separated further grid sizes to evaluate on, each with "
                         "held-out scenes of its own (2 scenes, 20 steps)")
    a = ap.parse_args(argv)
    gpu.load()
    if a.time_predict:
        out = {path: time_predict(a.time_predict, a.init, reps=2 if a.time_predict >= 256 else 10,
                                  tcgen05=path == "tcgen05") for path in ("tcgen05", "mma.sync")}
        print(json.dumps({"n": a.time_predict, "predict_ms": out,
                          "autotune": gpu.autotune_report().splitlines()}))
        return
    t0 = time.perf_counter()
    train_seeds = range(1000 + a.seed, 1000 + a.seed + a.scenes)
    hold_seeds = range(5000 + a.seed, 5000 + a.seed + a.holdout)
    data = collect(a.n, train_seeds, a.steps, a.every, keys=("A", "b", "x0", "r0", "x"))
    held = collect(a.n, hold_seeds, a.steps, a.every)
    t1 = time.perf_counter()
    net = gpu.UNet(seed=a.seed)
    if a.init:
        net.load(a.init)
    net.set_coarsening(a.coarsen)
    pres = [p for p in a.eval_precond.split(",") if p]
    rules = [r for r in a.eval_steps.split(",") if r]

    def evaluate_all(data, m):
        out = {}
        for rule in rules:
            os.environ["FLIPGPU_WARM_STEP"] = rule
            out[rule] = {p: evaluate(net, data, m, p) for p in pres}
        os.environ.pop("FLIPGPU_WARM_STEP", None)
        return out

    before = evaluate_all(held, a.n)
    hist = train(net, data, a.n, a.epochs, a.batch, a.lr, a.seed, log=print)
    t2 = time.perf_counter()
    n_train = int(data["A"].shape[0])
    del data
    after = evaluate_all(held, a.n)
    if a.out:
        net.save(a.out, trained_n=a.n, train_systems=n_train, epochs=a.epochs, batch=a.batch,
                 lr=a.lr)
    other = {}
    for m in [int(x) for x in a.eval_n.split(",") if x]:
        hm = collect(m, range(7000 + a.seed, 7002 + a.seed), 20, 5)
        other[m] = evaluate_all(hm, m)
        del hm
    print(json.dumps({"n": a.n, "train_systems": n_train,
                      "heldout_systems": int(held["A"].shape[0]), "collect_s": t1 - t0,
                      "train_s": t2 - t1, "loss": hist, "untrained": before, "trained": after,
                      "other_sizes": other}))


if __name__ == "__main__":
    main()

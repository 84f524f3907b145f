"""Trains the learned coarse-step corrector on solver-generated pairs and
deploys it with the plain-ETD judge (sclet_learned_step).

    python energy-stability_gb300/train_corrector.py train  --out corrector.npz [--N 64 --runs 200 ...]
    python energy-stability_gb300/train_corrector.py deploy --weights corrector.npz [--N 128 --steps 2000 ...]

Workload (beta->omega, plain ETD physics): four order parameters
U(-0.01, 0.01) from each run's seed, Landau 2-4-6, cubic elasticity, fine
dt 0.01, coarse dt 0.08 (ratio 8).

train: each run advances with the coarse step (mixed precision) from its
seeded state; at six seeded sample times between t = 0 and t = 150 the pair
(coarse step, eight fine FP64 steps) from the same state is recorded
(learned.make_pairs' normalisation).  Adam with cosine decay on mini-batches;
held-out runs give the error of the corrected coarse step relative to the
coarse step alone.  Writes the FP32 parameters and the record to --out.

deploy: --steps coarse steps at edge --N through sclet_learned_step (energy
and mass checks every step, deviation check every --check-every steps, fine
re-run on failure), beside the plain coarse run and the fine mixed-precision
run (rel L2 at checkpoints) and the fine FP64 run over the first --fp64-steps
coarse steps; throughput in cell-updates/s of the fine steps covered.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for _p in (HERE, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import learned  # noqa: E402
import sclet_gb300 as sg  # noqa: E402

RATIO = 8
DT = 0.01


def omega_case(seed: int, N: int):
    import cases
    return cases.Case(big_n=N, nac=4, nch=0, dt=DT, steps=1000, epn2=0.5, elastic=1, seed=seed, suffix="bo")


def sample_times(seed: int, count: int = 6, t_end: float = 150.0):
    """Seeded coarse-step counts, log-spread over [0, t_end]."""
    rng = np.random.default_rng(10_000 + seed)
    top = np.log1p(t_end / (DT * RATIO))
    steps = np.unique(np.round(np.expm1(np.sort(rng.uniform(0.0, top, count)))).astype(int))
    return [int(s) for s in steps]


def coarse_pairs(seeds, N: int, device: int = 0):
    """Pairs along coarse trajectories (see the module docstring)."""
    import torch
    xs, ys, ss = [], [], []
    fine = coarse = None
    for seed in seeds:
        case = omega_case(seed, N)
        if fine is None:
            fine = sg.Solver(learned.case_params(case), sg.FP64, device=device)
            coarse = sg.Solver(learned.case_params(case, dt=DT * RATIO), sg.MIXED, device=device)
        coarse.set_fields(learned.block_fields(case))
        k = 0
        for ks in sample_times(seed):
            if ks > k:
                coarse.step(ks - k)
                k = ks
            u = coarse.get_fields()
            coarse.step(1)
            k += 1
            uc = coarse.get_fields()
            fine.set_fields(u)
            fine.step(RATIO)
            uf = fine.get_fields()
            x, y, s = learned.pair(learned.owned(u), learned.owned(uc), learned.owned(uf))
            xs.append(torch.from_numpy(x).to(f"cuda:{device}"))
            ys.append(torch.from_numpy(y).to(f"cuda:{device}"))
            ss.append(s)
    fine.close()
    coarse.close()
    return torch.stack(xs), torch.stack(ys), np.array(ss)


def cmd_train(a):
    import torch
    t0 = time.time()
    X, Y, _ = coarse_pairs(range(a.runs), a.N)
    Xh, Yh, Sh = coarse_pairs(range(100_000, 100_000 + a.held_out), a.N)
    torch.cuda.synchronize()
    t1 = time.time()
    net = learned.Net(seed=a.seed, out_scale=1.0)
    losses = learned.train(net, X, Y, iters=a.iters, batch=a.batch, lr=a.lr)
    torch.cuda.synchronize()
    t2 = time.time()
    err = learned.relative_errors(net, Xh, Yh)
    agg = learned.aggregate_error(net, Xh, Yh, Sh)
    params = net.params()
    rec = {
        "workload": f"beta-omega {a.N}^3, 4 order parameters, Landau 2-4-6, elastic, fine dt {DT}, coarse dt "
                    f"{DT * RATIO}",
        "runs": a.runs, "pairs": int(X.shape[0]), "held_out_pairs": int(Xh.shape[0]),
        "iters": a.iters, "batch": a.batch, "lr": a.lr, "pair_seconds": t1 - t0, "train_seconds": t2 - t1,
        "seconds_per_iter": (t2 - t1) / a.iters,
        "loss_first": float(np.mean(losses[:20])), "loss_last": float(np.mean(losses[-100:])),
        "held_out_error_vs_coarse": agg,
        "held_out_pair_rel_error_median": float(np.median(err)),
        "note": "error vs coarse = |coarse + correction - fine| / |coarse - fine| summed over the held-out pairs in "
                "the fields' units; 1 is the coarse step alone.  Per pair the same ratio; pairs at rest (scale "
                "near the floor) make the mean of the per-pair ratio meaningless, hence the median",
    }
    np.savez(a.out, params=params, record=json.dumps(rec), losses=losses.astype(np.float32))
    print(json.dumps(rec), flush=True)
    net.close()


def _rel(u, v):
    own = (slice(None),) + (slice(2, -2),) * 3
    a, b = u[own], v[own]
    return [float(np.linalg.norm(a[f] - b[f]) / np.linalg.norm(b[f])) for f in range(a.shape[0])]


def cmd_deploy(a):
    import torch
    w = np.load(a.weights)
    case = omega_case(a.seed, a.N)
    u0 = learned.block_fields(case)
    pf, pc = learned.case_params(case), learned.case_params(case, dt=DT * RATIO)
    cells = a.N ** 3
    out = {"workload": f"beta-omega {a.N}^3, fine dt {DT}, coarse dt {DT * RATIO}, {a.steps} coarse steps",
           "training": json.loads(str(w["record"]))}
    checkpoints = sorted({int(c) for c in a.checkpoints.split(",") if int(c) <= a.steps} | {a.steps})
    # learned steps with the judge, and the plain coarse steps with the same judge
    runs = {}
    for name in ("learned", "coarse"):
        net = None
        if name == "learned":
            net = learned.Net(seed=1, out_scale=1.0)
            net.set_params(w["params"])
        coarse = sg.Solver(pc, sg.MIXED)
        fine = sg.Solver(pf, sg.MIXED)
        coarse.set_fields(u0)
        states, stats, secs = {}, None, 0.0
        done = 0
        for c in checkpoints:
            torch.cuda.synchronize()
            t = time.time()
            st = learned.learned_steps(coarse, fine, net, RATIO, c - done, check_every=a.check_every,
                                       deviation_bound=a.bound, energy_tol=a.energy_tol)
            secs += time.time() - t
            stats = st if stats is None else {k: (stats[k] + st[k] if k != "max_deviation" else
                                                  max(stats[k], st[k])) for k in st}
            done = c
            states[c] = coarse.get_fields()
        runs[name] = (states, stats, secs)
        for s in (coarse, fine):
            s.close()
        if net:
            net.close()
    # fine references
    fine = sg.Solver(pf, sg.MIXED)
    fine.set_fields(u0)
    ref, done, fsecs = {}, 0, 0.0
    for c in checkpoints:
        torch.cuda.synchronize()
        t = time.time()
        fine.step(RATIO * (c - done))
        fine.sync()
        fsecs += time.time() - t
        done = c
        ref[c] = fine.get_fields()
    fine.close()
    f64 = sg.Solver(pf, sg.FP64)
    f64.set_fields(u0)
    t = time.time()
    f64.step(RATIO * a.fp64_steps)
    f64.sync()
    f64_secs = time.time() - t
    ref64 = f64.get_fields()
    f64.close()
    # the learned and coarse runs at the FP64 horizon
    extra = {}
    for name in ("learned", "coarse"):
        net = None
        if name == "learned":
            net = learned.Net(seed=1, out_scale=1.0)
            net.set_params(w["params"])
        coarse = sg.Solver(pc, sg.MIXED)
        fine = sg.Solver(pf, sg.MIXED)
        coarse.set_fields(u0)
        learned.learned_steps(coarse, fine, net, RATIO, a.fp64_steps, check_every=a.check_every,
                              deviation_bound=a.bound, energy_tol=a.energy_tol)
        extra[name] = coarse.get_fields()
        for s in (coarse, fine):
            s.close()
        if net:
            net.close()
    for name, (states, stats, secs) in runs.items():
        out[name] = {
            "stats": stats, "fallback_rate": stats["fallbacks"] / max(stats["steps"], 1), "seconds": secs,
            "cell_updates_per_s": cells * RATIO * a.steps / secs,
            "coarse_cell_updates_per_s": cells * a.steps / secs,
            "rel_l2_vs_fine_mixed": {str(c): _rel(states[c], ref[c]) for c in checkpoints},
            "rel_l2_vs_fine_fp64": {"coarse_steps": a.fp64_steps, "per_field": _rel(extra[name], ref64)},
        }
    out["fine_mixed"] = {"seconds": fsecs, "cell_updates_per_s": cells * RATIO * a.steps / fsecs}
    out["fine_fp64"] = {"fine_steps": RATIO * a.fp64_steps, "seconds": f64_secs,
                        "cell_updates_per_s": cells * RATIO * a.fp64_steps / f64_secs}
    out["speedup_learned_vs_fine_fp64"] = out["learned"]["cell_updates_per_s"] / out["fine_fp64"]["cell_updates_per_s"]
    out["speedup_learned_vs_fine_mixed"] = out["learned"]["cell_updates_per_s"] / out["fine_mixed"]["cell_updates_per_s"]
    print(json.dumps(out), flush=True)
    if a.json:
        with open(a.json, "w") as fp:
            json.dump(out, fp, indent=1)


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--out", required=True)
    t.add_argument("--N", type=int, default=64)
    t.add_argument("--runs", type=int, default=200)
    t.add_argument("--held-out", type=int, default=10)
    t.add_argument("--iters", type=int, default=3000)
    t.add_argument("--batch", type=int, default=4)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--seed", type=int, default=5)
    d = sub.add_parser("deploy")
    d.add_argument("--weights", required=True)
    d.add_argument("--N", type=int, default=128)
    d.add_argument("--steps", type=int, default=2000)
    d.add_argument("--checkpoints", default="250,500,1000,1500")
    d.add_argument("--check-every", type=int, default=50)
    d.add_argument("--bound", type=float, default=2e-2)
    d.add_argument("--energy-tol", type=float, default=1e-9)
    d.add_argument("--fp64-steps", type=int, default=125)
    d.add_argument("--seed", type=int, default=7777)
    d.add_argument("--json", default="")
    a = ap.parse_args()
    {"train": cmd_train, "deploy": cmd_deploy}[a.cmd](a)


if __name__ == "__main__":
    main()

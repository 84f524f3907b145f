"""Benchmark of the ScLETD ETD step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64]
                    [--impl reference] [--size N3EDGE] [--accuracy-steps S]

Workload: the beta->alpha coupled case -- one conserved concentration
c = 0.5 + U(-0.02, 0.02) and four order parameters U(-0.01, 0.01) on a 512^3
periodic grid (block edge 516; --size 192 gives the 192^3 case), Landau 2-4-6 with cross term 1.5 and c-eta
coupling 0.8, anisotropic gradient tensors diag(0.5, 0.5, 0.3) with
stabiliser kk = 0.5, cubic elasticity C11/C12/C44 = 1.0/0.6/0.4 with four
<111> eigenstrains, dt = 0.005, first-order ETD.  Synthetic seeded data.

A step is one pass of the reference's time loop (ghost exchange, elastic
force, right-hand sides, eigenbasis transforms and update) plus the
diagnostics check_soln_new it runs every pass, all inside the timed region.  `value` is cell-updates/s
(N^3 owned cells x steps / time) of the mixed-precision step (default) with
the state resident in HBM; `e2e` is the same through the C ABI with the
fields copied in from pinned host memory and copied back out (with the
diagnostics) every step.  The plain FP64 step is timed beside it ("fp64"),
and "accuracy_vs_fp64" compares the two forms after --accuracy-steps steps
from the same state.

--impl reference times the reference's CPU path (the C restatement of
oracle/, the reference's own build cannot run on this host) on all host
cores, on the same workload.  A 512^3 step takes minutes on the host, so the
CPU sample is bounded by time: it reports the steps it actually timed and
the per-step rate is extrapolated from them.

Several GPUs (torchrun): independent replicas with their own seeds (the path
has no data exchange between replicas); value = all ranks' cell updates /
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "energy-stability_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import cases  # noqa: E402

METRIC = "cell-updates/s on 1 GB300: mixed/learned vs plain FP64 at ≤1e-5 rel L2"
UNIT = "cell-updates/s"
# DRAM bytes (read + write) of one tensor-core product launch over its
# algorithmic bytes, from an ncu capture of a ten-tensor launch at 192^3:
# (692.4 + 273.6) MB over 10 x 196^3 x (8 + 4) B = 903.6 MB.
TC_TRAFFIC_RATIO = 1.069
FP64_PEAK_TFLOPS = 1.25  # nominal GB300 FP64 rate (the measured peaks cover HBM and bf16 only)


def workload(big_n: int, seed: int) -> cases.Case:
    return cases.Case(
        big_n=big_n, nac=4, nch=1, etd2=0, elastic=1, anisotropic=1, kk=(0.5, 0.5, 0.5),
        lambdas=[np.diag([0.5, 0.5, 0.3]) for _ in range(4)], dt=0.005, epn2=1.0, steps=2000,
        eta_range=(-0.01, 0.01), c_range=(0.48, 0.52), seed=seed, suffix="bench")


ENSEMBLE_EDGES = (32, 48, 64, 80, 96)


def ensemble_case(edge: int, seed: int, a2: float) -> cases.Case:
    """One run of the batched beta->omega ensemble: four order parameters
    U(-0.01, 0.01) from its seed, Landau 2-4-6 with its own a2, cubic
    elasticity, dt 0.01."""
    landau = list(cases.Case().landau)
    landau[0] = a2
    return cases.Case(big_n=edge, nac=4, nch=0, dt=0.01, steps=500, epn2=0.5, elastic=1, seed=seed,
                      landau=tuple(landau), suffix="ens")


def ensemble_runs(count: int = 256, seed: int = 2026):
    """The ensemble's runs: (edge, seed, a2) with edges drawn from
    ENSEMBLE_EDGES and a2 ~ U(-1.2, -0.8), seeded."""
    rng = np.random.default_rng(seed)
    edges = rng.choice(ENSEMBLE_EDGES, size=count)
    a2 = rng.uniform(-1.2, -0.8, size=count)
    return [(int(e), 10_000 + i, float(a)) for i, (e, a) in enumerate(zip(edges, a2))]


def case_params(sg, case):
    with tempfile.TemporaryDirectory() as td:
        cases.write_case(case, td, eigen=False, fields=False)
        return sg.read_case(td, case.suffix)


def workload_name(big_n: int) -> str:
    return (f"beta-alpha coupled CH + 4 AC, {big_n}^3 periodic (block {big_n + 4}^3), Landau 2-4-6, "
            f"anisotropic, cubic elasticity, ETD1, dt 0.005")


def config_of(big_n: int, world: int) -> dict:
    return {"workload": workload_name(big_n), "cells_per_step": big_n ** 3,
            "l2": "inputs larger than L2 (state of a step > 129 MB)", "parallelism": f"replicas x{world}"}


def block_fields(case: cases.Case) -> np.ndarray:
    n = case.n
    out = np.zeros((case.nac + case.nch, n, n, n))
    for f, (_, _, vals) in enumerate(case.initial_fields()):
        out[f, 2:-2, 2:-2, 2:-2] = vals
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.out = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=10)

    def summary(self):
        try:
            with open(self.out.name) as fp:
                rows = [r.split(",") for r in fp.read().strip().splitlines() if r.strip()]
        except Exception:
            rows = []
        os.unlink(self.out.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and "Active" in r[5 + i]
                          and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    """Replica ranks from the torchrun environment: NCCL with one GPU per rank,
    gloo where no GPU is visible (host-side runs of the same code)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
    return world, rank, local


def dist_max(x: float, world: int) -> float:
    """Maximum over ranks (the slowest replica's time)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_oracle_rate(case: cases.Case, steps: int, warmup: int, budget_s: float = 120.0):
    """Times the C oracle (all host threads) on the case: `warmup` untimed
    steps (at most one), then up to `steps` timed steps with the diagnostics
    of each, stopping once `budget_s` seconds are spent (the sample is then
    shorter than `steps`).  Returns (cell-updates/s, cores, seconds, steps
    timed)."""
    import oracle_py
    if not os.path.exists(oracle_py.LIB_PATH):
        oracle_py.build()
    with tempfile.TemporaryDirectory() as td:
        cases.write_case(case, td, fields=False)
        p = oracle_py.load_case_params(td, case.suffix, block_fields(case))
        o = oracle_py.Oracle(p)
        o.step(min(warmup, 1))
        done, dt = 0, 0.0
        while done < max(steps, 1) and (done == 0 or dt < budget_s):
            t0 = time.perf_counter()
            o.step(1)
            o.check_soln()
            dt += time.perf_counter() - t0
            done += 1
    return case.big_n ** 3 * done / dt, o.threads(), dt, done


def cpu_budget(size: int) -> tuple[int, float]:
    """Warm-up steps and time budget of a CPU sample: a 512^3 step takes a
    few minutes on 16 host threads, so large grids time one step, no warm-up."""
    return (0, 1.0) if size >= 384 else (1, 120.0)


def sample_text(done: int, asked: int, warm: int, cores: int, secs: float) -> str:
    cut = f", {done} of {asked} asked, per-step rate extrapolated from them" if done < asked else ""
    return (f"{done} full step(s) of the workload with diagnostics{cut}, after {warm} warm-up step(s) "
            f"(C restatement of the reference's step, OpenMP on {cores} threads, {secs:.1f} s)")


def run_reference(args, world, rank):
    if rank != 0:
        return
    case = workload(args.size, seed=1000)
    warm, budget = cpu_budget(args.size)
    warm = min(warm, args.warmup)
    rate, cores, secs, done = cpu_oracle_rate(case, args.steps, warm, budget)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": world,
        "steps": done, "warmup": warm, "ms_per_step": 1000.0 * secs / done,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(args.size, world),
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample_text(done, args.steps, warm, cores, secs)},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


STAGES = ["products", "rhs", "elastic", "halo", "diagnostics", "tc_kernel", "slicing"]


def peaks(sustained=False):
    """Measured HBM copy bandwidth and bf16 GEMM throughput of this GPU model
    (MEASURED_PEAKS.json beside this file; the bf16 figure as a burst, or
    sustained over seconds under the power cap), else the earlier GB300
    figures."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fp:
            d = json.load(fp)
        bf16 = float(d["bf16_tflops_sustained"] if sustained else d["bf16_tflops"])
        return float(d["hbm_gbs"]), bf16, "measured (MEASURED_PEAKS.json" + (", sustained bf16)" if sustained else ")")
    except Exception:
        return 6800.0, 1700.0 if sustained else 1900.0, "fallback (no MEASURED_PEAKS.json)"


def timed_steps(s, steps, world, local):
    """K steps, each bracketed by CUDA events on the context's stream.  The
    context queues the diagnostics (check_soln_new, which the reference runs
    after every pass) inside each step; the host reads each record between
    steps, outside the timed brackets."""
    dist_barrier(world)
    l0 = s.launch_count()
    with ClockSampler(local) as clk:
        s.sync()
        ms = 0.0
        for _ in range(steps):
            ms += s.time_steps(1)
            s.last_diagnostics()
    return ms, s.launch_count() - l0, clk.summary()


def profiled_stages(s, steps=2):
    s.set_profiling(True)
    s.time_steps(steps)
    ms, launches = s.stage_times(len(STAGES))
    s.set_profiling(False)
    return dict(zip(STAGES, ms)), dict(zip(STAGES, launches))


def tc_mma_flops(n):
    """Physical BF16 MMA flops of one split product (n x n matrix times an n^3
    tensor) as the tensor-core kernel issues them: eleven MMAs per k-step of
    16, input rows padded to 128-row tiles (M), the eigen-modes in 128-wide
    tiles with the last one N = its live modes rounded up to 16, and k-steps
    over the 32-wide k-blocks with the last k-block's second k-step skipped
    when it holds only zero columns."""
    r_pad = (n * n + 127) // 128 * 128
    full, last = divmod(n, 128)
    a_eff = 128 * full + ((last + 15) // 16 * 16 if last else 0)
    nkb = (n + 31) // 32
    ksteps = 2 * (nkb - 1) + (2 if n - 32 * (nkb - 1) > 16 else 1)
    return 11 * 2.0 * r_pad * a_eff * 16 * ksteps


def tc_roofline(case, stage_ms, stage_launches, steps):
    """Roofline of the tensor-core mode-n product kernel over `steps` profiled
    steps.  The kernel is bound by the tensor pipe: `achieved` counts the
    physical BF16 MMA flops of the split product (tc_mma_flops) over its live
    CUDA-event time, against the measured sustained bf16 rate (the kernel runs
    inside a long step); the algorithmic flops (2 n^4 per product) are
    `algorithmic_tflops`.  The HBM view (`hbm`): the bytes the kernel must
    move given its interface, the four BF16 slice planes of the input (8 B per
    element; the zero columns up to the next multiple of 32 are not counted)
    and the FP32 output (4 B per element), plus, for the fused ETD update of
    one product in nine, the other operand (4 B) and the coefficient pairs
    (16 B)."""
    n, F = case.n, case.nac + case.nch
    per_step_products = 9 * F
    elems = n ** 3
    bytes_step = per_step_products * elems * (8.0 + 4.0) + F * elems * 20.0
    flops_step = per_step_products * 2.0 * n ** 4
    mma_step = per_step_products * tc_mma_flops(n)
    t = stage_ms["tc_kernel"] / 1000.0
    launches = max(stage_launches["tc_kernel"], 1)
    per_launch = bytes_step * steps / launches
    hbm, bf16s, src = peaks(sustained=True)
    _, bf16b, _ = peaks()
    gbs = bytes_step * steps / t / 1e9
    mma = mma_step * steps / t / 1e12
    return {
        "bound": "tensor", "kernel": "modeprod_tc_kernel (split-BF16 tcgen05 eigenbasis products)",
        "achieved": mma, "peak": bf16s, "unit": "TFLOP/s", "frac": mma / bf16s,
        "achieved_counts": "physical BF16 MMA flops of the split product (eleven MMAs per term)",
        "frac_of_burst_peak": mma / bf16b, "algorithmic_tflops": flops_step * steps / t / 1e12,
        "traffic": per_launch * TC_TRAFFIC_RATIO,
        "traffic_source": f"ncu DRAM read+write / algorithmic bytes = {TC_TRAFFIC_RATIO} on one 192^3 launch of ten "
                          "tensors (--set full capture), scaled to this launch size",
        "peak_source": src, "avg_launch_ms": stage_ms["tc_kernel"] / launches,
        "hbm": {"achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                "algorithmic_bytes_per_launch": per_launch, "bytes_per_step": bytes_step},
    }


def fp64_stage_roofline(case, stage_ms_per_step):
    """HBM fraction of the plain FP64 step's stencil, FFT and diagnostics
    stages on their algorithmic bytes per cell-update (owned cell, all
    fields): right-hand sides 8 F (read the fields) + 8 nac (elastic force) +
    8 F (write) B; elastic force 112 B per order parameter (forward R2C and
    inverse C2R, three axis passes reading and writing half a complex value
    each, plus the real field in and out); diagnostics 8 F B."""
    hbm, _, src = peaks()
    F, nac = case.nac + case.nch, case.nac
    cells = case.big_n ** 3
    per_cell = {"rhs": 16.0 * F + 8.0 * nac, "elastic": 112.0 * nac, "diagnostics": 8.0 * F}
    out = {}
    for k, b in per_cell.items():
        ms = stage_ms_per_step.get(k, 0.0)
        if ms > 0:
            gbs = b * cells / (ms / 1000.0) / 1e9
            out[k] = {"bytes_per_cell": b, "ms": ms, "gbs": gbs, "frac": gbs / hbm}
    out["peak"] = hbm
    out["peak_source"] = src
    return out


def ensemble_bench(sg, local, steps: int, loop_steps: int = 5, count: int = 256):
    """The batched ensemble: `count` runs (edges drawn from 32..96, own seeds
    and a2) as one context per edge holding its runs side by side, tuned by
    the autotuner, stepped by one captured graph over all edges; against the
    single-run path looped over the runs (one context per run, ordinary
    steps).  Device time (CUDA events) of `steps` ensemble steps and of
    `loop_steps` steps of every single run; cell-updates/s over all runs."""
    runs = ensemble_runs(count)
    groups = {}
    for edge, seed, a2 in runs:
        groups.setdefault(edge, []).append((seed, a2))
    solvers, tuned = [], {}
    for edge in sorted(groups):
        members = groups[edge]
        p = case_params(sg, ensemble_case(edge, members[0][0], members[0][1]))
        u0 = np.concatenate([block_fields(ensemble_case(edge, sd, a)) for sd, a in members])
        s = sg.Solver(p, sg.MIXED, device=local, runs=len(members), krun=np.array([a for _, a in members]))
        s.set_fields(u0)
        s.step(1)
        tuned[edge] = s.tune(2)
        solvers.append(s)
    cells = sum(e ** 3 for e, _, _ in runs)
    ens = sg.Ensemble(solvers)
    ens.step(3)
    ens.sync()
    ms = ens.time_steps(steps)
    diag_ok = all(np.isfinite(s.check_soln(1)).all() for s in solvers)
    ens.close()
    for s in solvers:
        s.close()
    # the single-run path, looped
    loop_ms = 0.0
    for edge, seed, a2 in runs:
        case = ensemble_case(edge, seed, a2)
        s = sg.Solver(case_params(sg, case), sg.MIXED, device=local)
        s.set_fields(block_fields(case))
        s.step(2)
        loop_ms += s.time_steps(loop_steps)
        s.close()
    batched = cells * steps / (ms / 1000.0)
    looped = cells * loop_steps / (loop_ms / 1000.0)
    return {
        "workload": f"{count} beta-omega runs, edges {list(ENSEMBLE_EDGES)} (seeded), own seed and a2 U(-1.2,-0.8), "
                    "4 order parameters, elastic, dt 0.01, FP32 fields / FP64 energy",
        "runs_per_edge": {str(e): len(groups[e]) for e in sorted(groups)},
        "cells_per_step": cells, "steps": steps, "ms_per_step": ms / steps,
        "value": batched, "unit": UNIT,
        "looped_single_run": {"value": looped, "steps_per_run": loop_steps, "ms_per_step_all_runs": loop_ms / loop_steps},
        "speedup_vs_looped": batched / looped,
        "tuned": {str(e): {"rhs_zplanes": z, "tc_ctas": c} for e, (z, c) in tuned.items()},
        "diagnostics_finite": bool(diag_ok),
    }


def accuracy_check(sg, params, u0, steps, every, local):
    """Mixed against FP64 from the same state: at every `every` steps up to
    `steps`, relative L2 per field over the owned cells, the energy (pointwise
    and as |dE| / max|E| over the curve so far) and the relative difference of
    each field's volume integral (the conserved field's mass)."""
    if steps <= 0:
        return None
    every = every if every > 0 else steps
    a = sg.Solver(params, sg.FP64, device=local)
    b = sg.Solver(params, sg.MIXED, device=local)
    for x in (a, b):
        x.set_fields(u0)
    own = (slice(2, -2),) * 3
    e64, e32, rows = [a.check_soln()[0, 3]], [b.check_soln()[0, 3]], []
    done = 0
    while done < steps:
        k = min(every, steps - done)
        a.step(k)
        b.step(k)
        done += k
        ua, ub = a.get_fields(), b.get_fields()
        da, db = a.check_soln(), b.check_soln()
        e64.append(da[0, 3])
        e32.append(db[0, 3])
        rel = [float(np.linalg.norm(ub[f][own] - ua[f][own]) / np.linalg.norm(ua[f][own])) for f in range(ua.shape[0])]
        rows.append({"step": done, "field_rel_l2": rel,
                     "energy_rel": float(abs(db[0, 3] - da[0, 3]) / abs(da[0, 3])),
                     "energy_curve_rel": float(np.max(np.abs(np.array(e32) - np.array(e64))) / np.max(np.abs(e64))),
                     "volume_rel": [float(abs(db[f, 2] - da[f, 2]) / abs(da[f, 2])) for f in range(ua.shape[0])],
                     "max_abs_eta": float(np.abs(ua[0][own]).max())})
    a.close()
    b.close()
    last = rows[-1]
    return {"steps": steps, "max_field_rel_l2": max(last["field_rel_l2"]),
            "energy_curve_rel": max(r["energy_curve_rel"] for r in rows), "checkpoints": rows}


def run_gpu(args, world, rank, local):
    import sclet_gb300 as sg
    sg.lib()
    precision = {"fp64": sg.FP64, "mixed": sg.MIXED}[args.precision]
    case = workload(args.size, seed=1000 + rank)
    n, F = case.n, case.nac + case.nch
    with tempfile.TemporaryDirectory() as td:
        cases.write_case(case, td, eigen=False, fields=False)
        params = sg.read_case(td, case.suffix)
    u0 = block_fields(case)
    s = sg.Solver(params, precision, device=local)
    s.set_step_diagnostics(1)
    s.set_fields(u0)
    s.step(args.warmup)
    s.last_diagnostics()
    # device-resident timed region
    ms, launches, clocks = timed_steps(s, args.steps, world, local)
    ms_max = dist_max(ms, world)
    cells = case.big_n ** 3 * args.steps * world
    value = cells / (ms_max / 1000.0)
    # end to end through the C ABI with host buffers: every step copies all
    # fields in from pinned memory, steps, reads the diagnostics and copies
    # all fields back out.  The copies are queued on the copy streams, so the
    # next step's inputs cross the host link while this step runs.
    pin_in = sg.PinnedArray((F, n, n, n))
    pin_out = sg.PinnedArray((F, n, n, n))
    pin_in.array[...] = u0
    dist_barrier(world)
    s.sync()
    t0 = time.perf_counter()
    s.set_fields_async(pin_in.array)
    for k in range(args.steps):
        s.step(1)
        s.get_fields_async(pin_out.array)
        if k + 1 < args.steps:
            s.set_fields_async(pin_in.array)
        s.last_diagnostics()
    s.sync()
    e2e_s = dist_max(time.perf_counter() - t0, world)
    if not np.isfinite(pin_out.array).all():
        raise RuntimeError("end-to-end results are not finite")
    e2e_value = cells / e2e_s
    bytes_step = F * n ** 3 * 8
    pin_in.free()
    pin_out.free()
    stage_ms, stage_launches = profiled_stages(s, 2)
    s.close()
    # the CPU baseline runs on the host cores while the GPU times the plain
    # FP64 step (whose kernels last tens to thousands of milliseconds, so the
    # launching thread sharing the cores costs it nothing)
    cpu_box = {}
    cpu_thread = None
    if not args.no_cpu_baseline and world == 1:
        def cpu_leg():
            small = workload(args.size, seed=1000)
            warm, budget = cpu_budget(args.size)
            cpu_box["r"] = cpu_oracle_rate(small, args.cpu_steps, warm, budget)
        cpu_thread = threading.Thread(target=cpu_leg, daemon=True)
        cpu_thread.start()
    # the plain FP64 step beside it (same workload, same timing)
    fp64 = None
    if precision == sg.MIXED and not args.no_fp64:
        s64 = sg.Solver(params, sg.FP64, device=local)
        s64.set_step_diagnostics(1)
        s64.set_fields(u0)
        s64.step(args.warmup)
        ms64, _, _ = timed_steps(s64, args.steps, world, local)
        st64, _ = profiled_stages(s64, 1)
        s64.close()
        ms64 = dist_max(ms64, world)
        fp64 = {"value": cells / (ms64 / 1000.0), "ms_per_step": ms64 / args.steps,
                "speedup_of_mixed": ms64 / ms_max, "stage_ms_per_step": st64,
                "stage_hbm": fp64_stage_roofline(case, st64)}
    ensemble = None
    if precision == sg.MIXED and rank == 0 and args.ensemble_steps > 0:
        ensemble = ensemble_bench(sg, local, args.ensemble_steps)
    accuracy = None
    if precision == sg.MIXED and rank == 0:
        acc_steps = args.accuracy_steps if args.accuracy_steps is not None else (10 if args.size >= 384 else 100)
        accuracy = accuracy_check(sg, params, u0, acc_steps, args.accuracy_every, local)
    cpu = None
    if cpu_thread is not None:
        cpu_thread.join()
        rate, cores, secs, done = cpu_box["r"]
        warm = cpu_budget(args.size)[0]
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": sample_text(done, args.cpu_steps, warm, cores, secs)
               + "; run on the host while the GPU timed the FP64 step"}
    if rank != 0:
        return
    if precision == sg.MIXED:
        roofline = tc_roofline(case, stage_ms, stage_launches, 2)
    else:
        flops_products = 2.0 * n ** 4 * 9 * F * 2
        achieved = flops_products / (stage_ms["products"] / 1000.0) / 1e12
        roofline = {"bound": "fp64", "kernel": "modeprod_f64 (eigenbasis mode-n products)", "achieved": achieved,
                    "peak": FP64_PEAK_TFLOPS, "unit": "TFLOP/s", "frac": achieved / FP64_PEAK_TFLOPS, "traffic": None,
                    "peak_source": "nominal GB300 FP64",
                    "avg_launch_ms": stage_ms["products"] / max(stage_launches["products"], 1)}
    roofline["stage_ms_per_step"] = {k: v / 2 for k, v in stage_ms.items()}
    roofline["stage_launches_per_step"] = {k: v // 2 for k, v in stage_launches.items()}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if precision == sg.FP64 else "bf16-slices/f32 (f64 eigenbasis, diagnostics, mass)",
        "data": "synthetic",
        "config": config_of(args.size, world), "precision": args.precision,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": bytes_step, "d2h_bytes_per_step": bytes_step},
        "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
        "fp64": fp64, "accuracy_vs_fp64": accuracy, "ensemble": ensemble,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--size", type=int, default=512, help="physical grid edge N")
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip timing the plain FP64 step beside the mixed one")
    ap.add_argument("--accuracy-steps", type=int, default=None,
                    help="steps of the mixed-vs-FP64 check from the same state (0: skip; default 10 at 512^3, "
                         "100 below)")
    ap.add_argument("--accuracy-every", type=int, default=0, help="checkpoint interval of that check (0: end only)")
    ap.add_argument("--ensemble-steps", type=int, default=500,
                    help="timed steps of the batched 256-run ensemble beside the headline (0: skip)")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: start the replicas under torchrun
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr=127.0.0.1", f"--master-port={29500 + os.getpid() % 1000}",
               os.path.abspath(__file__), *sys.argv[1:]]
        sys.exit(subprocess.call(cmd))
    world, rank, local = dist_setup()
    if world != args.gpus:
        raise SystemExit(f"--gpus {args.gpus} but the launcher started {world} ranks")
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

#!/usr/bin/env python3
"""Benchmark of the GB300 PLSQR3 hot path: the LSQR iteration and its aprod.

Workload: the 96x96x32-cell tomography problem (294,912 columns, 200,000 rays
of radius-6 tubes, ~1.33e9 kernel nonzeros, 1,148,928 damping rows), plain
FP64 LSQR for 300 iterations.  One step = one LSQR solve with the matrix
resident in HBM.

  value  = algorithmic HBM bytes of the solve's main loop / its device time
           (CUDA events on the solver's stream around the iteration loop)
  e2e    = the same bytes / wall time of the whole plsqr_lsqr call with host
           b_k in and host x out (H2D and D2H inside the timed region)

Extra keys: roofline of the dominant kernel (the slower product), the CPU
baseline (the oracle port, FP64, all host threads, the iteration loop of a
bounded sample, CPU model), the time to 1e-6 relative error vs the FP64
solution for plain FP64 and mixed precision (one sweep; the configuration's
50 iterations per sweep; FP32 vectors as well), the learned warm start +
mixed precision against both on held-out instances (network trained in the
run on a bounded set of pairs, --warm-train), clocks sampled during the
timed region.

`--impl reference` times the reference CPU implementation of the same solve
(the oracle port of source/lsqr.c + aprod_impl.c + CPUSpMV.c, OpenMP on all
host cores) on a bounded sample and prints the same metric.

`--extension batched|uneven|warm` measures an extension instead (one JSON
line each): 32 right-hand sides on the 96x96x32 operator against the plain
path run once per right-hand side; the 24 uneven problems in one persistent
launch against the one-problem path; the learned warm start (2,000 training
pairs, training, iterations and time to 1e-6 on held-out seeds, cold
against warm).  `--profile` runs one short case of the chosen path for ncu.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import __graft_entry__ as graft  # noqa: E402

METRIC = "aprod HBM GB/s (plain FP64 LSQR iteration)"
UNIT = "GB/s"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel: str):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "aprod_fp64_grid96.md"
    if not p.exists():
        return None
    m = re.search(rf"^{kernel}_dram_bytes_per_launch:\s*([0-9.eE+]+)", p.read_text(), re.M)
    return float(m.group(1)) if m else None


class Clocks:
    """nvidia-smi sampling (every 200 ms) during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else platform)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_sample(pkg, orc, prob, iterations: int) -> dict:
    """The oracle port (FP64, OpenMP on every host thread) on `iterations`
    LSQR iterations of the same problem, timed over the iteration loop only:
    the region of the reference's own "Parallel LSQR time" (source/lsqr.c:
    476-478, 836-842), start-up excluded."""
    o = orc.OracleProblem(prob)
    threads = orc.get_threads()
    t0 = time.perf_counter()
    r = o.lsqr(iterations)
    wall = time.perf_counter() - t0
    return dict(seconds=r["result"]["loop_seconds"], wall_seconds=wall, iterations=iterations,
                threads=threads)


def cpu_sample_text(cfg: str, iterations: int, steps: int = 1) -> str:
    return (f"{steps} x {iterations} LSQR iterations of the {cfg} solve, timed over the "
            f"iteration loop only (the reference's 'Parallel LSQR time' region, start-up "
            f"excluded); host CPU {cpu_model()}")


def max_over_ranks(values: list[float]) -> list[float]:
    """Element-wise maximum over the ranks of an initialised process group
    (the replicas' times); the values themselves on a single process."""
    try:
        import torch.distributed as tdist
        if not (tdist.is_available() and tdist.is_initialized()):
            return list(values)
        import torch
    except ImportError:
        return list(values)
    t = torch.tensor(values, dtype=torch.float64)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return [float(v) for v in t]


def first_below(err: np.ndarray, tol: float):
    idx = np.nonzero((err >= 0) & (err <= tol))[0]
    return int(idx[0]) if idx.size else None


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="grid96")
    ap.add_argument("--iterations", type=int, default=None)
    ap.add_argument("--cpu-iterations", type=int, default=5,
                    help="LSQR iterations of each CPU baseline sample (loop timed alone)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tts", action="store_true", help="skip the time-to-1e-6 runs")
    ap.add_argument("--warm-train", type=int, default=64,
                    help="default run: training pairs of the warm-start network (0: skip)")
    ap.add_argument("--warm-epochs", type=int, default=6)
    ap.add_argument("--warm-eval", type=int, default=2,
                    help="default run: held-out instances timed to 1e-6 in the three forms")
    ap.add_argument("--profile", action="store_true",
                    help="profiling run: build the context, run one short solve, exit")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--train", type=int, default=2000, help="warm start: training pairs")
    ap.add_argument("--epochs", type=int, default=6, help="warm start: passes over the pairs")
    ap.add_argument("--heldout", type=int, default=200, help="warm start: held-out seeds")
    ap.add_argument("--timed-single", type=int, default=4,
                    help="warm start: held-out seeds also timed one at a time")
    ap.add_argument("--timed", type=int, default=16,
                    help="warm start: held-out seeds timed to 1e-6 against FP64 references")
    ap.add_argument("--extension", default=None, choices=["batched", "uneven", "warm"],
                    help="measure an extension instead: 32 right-hand sides on the "
                         "96x96x32 operator, the 24 uneven problems in one launch, or the "
                         "learned warm start (training set, training, held-out iterations)")
    ap.add_argument("--variant-rows", type=int, default=-1,
                    help="batched product variant of A x (-1: pick by timing)")
    ap.add_argument("--variant-cols", type=int, default=-1,
                    help="batched product variant of A^T y (-1: pick by timing)")
    ap.add_argument("--rhs", type=int, default=32,
                    help="batched profiling run: right-hand sides (the first of the 32)")
    args = ap.parse_args()

    ws, rank, local = dist()
    pkg = graft.load_package()
    if args.extension and not args.profile:
        if rank != 0:
            return 0
        fn = {"batched": bench_batched, "uneven": bench_uneven, "warm": bench_warm}[args.extension]
        print(json.dumps(fn(pkg, args, local)))
        return 0
    cfg = pkg.CONFIGS[args.config]
    iters = args.iterations or cfg["iterations"]

    if args.impl == "reference":
        if rank != 0:
            return 0
        orc = graft.load_oracle()
        log(f"generating {args.config} ...")
        prob = pkg.generate(args.config)
        bytes_it = algorithmic_bytes(prob)
        per = []
        for _ in range(min(args.warmup, 1)):
            cpu_sample(pkg, orc, prob, 1)
        for _ in range(args.steps):
            s = cpu_sample(pkg, orc, prob, args.cpu_iterations)
            per.append(s)
        secs = sum(s["seconds"] for s in per)
        its = sum(s["iterations"] for s in per)
        value = bytes_it * its / secs / 1e9
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
                "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded generator, reference file formats)",
                "config": workload(args.config, prob, iters),
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": per[0]["threads"],
                                 "kind": "port", "cpu_model": cpu_model(),
                                 "seconds_per_iteration": secs / its,
                                 "loop_seconds": secs,
                                 "wall_seconds_with_startup": sum(s["wall_seconds"] for s in per),
                                 "sample": cpu_sample_text(args.config, args.cpu_iterations,
                                                           args.steps)},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    if args.profile and args.extension == "batched":
        prob = pkg.generate(args.config)
        with pkg.Context(prob, device=local) as ctx:
            insts = pkg.batch.instances(ctx, prob, args.config)[:args.rhs]
            out = ctx.batch_lsqr(np.stack([i.b_k for i in insts]), lam=[i.lam for i in insts],
                                 sweeps=1, inner=2, variant_rows=args.variant_rows,
                                 variant_cols=args.variant_cols)
        log(f"profile run: {args.config}, {len(insts)} right-hand sides, variants {out['info']}")
        return 0
    if args.profile and args.extension == "uneven":
        probs = [pkg.generate(c) for c in pkg.multi.uneven_configs()]
        with pkg.multi.Multi(probs, device=local) as mp:
            out = mp.solve()
        log(f"profile run: 24 uneven problems, {out['seconds'] * 1e3:.2f} ms")
        return 0
    if args.profile and args.extension == "warm":
        # the network alone on the 96x96x32 grid: three training steps and a
        # prediction on seeded volumes (no operator needed)
        grid = (96, 96, 32)
        rng = np.random.default_rng(5)
        z = rng.standard_normal(96 * 96 * 32).astype(np.float32)
        with pkg.warm.UNet(grid, seed=1, device=local) as net:
            for _ in range(3):
                net.train_step(z, np.roll(z, 1), 1e-3)
            net.predict(z)
        log("profile run: U-Net 96x96x32, 3 training steps + 1 prediction")
        return 0
    if args.profile:
        prob = pkg.generate(args.config)
        with pkg.Context(prob, device=local, precision=args.precision) as ctx:
            if args.precision == "mixed":
                out = ctx.lsqr(sweeps=1, inner=iters)
            else:
                out = ctx.lsqr(lsqr_iteration=iters)
        log(f"profile run: {args.config}, {iters} iterations, "
            f"{out['result']['seconds'] * 1e3:.2f} ms")
        return 0

    # ---- GB300 arm ----------------------------------------------------------
    if ws > 1:
        import torch.distributed as tdist
        tdist.init_process_group("gloo")
    log(f"[rank {rank}] generating {args.config} ...")
    t0 = time.perf_counter()
    prob = pkg.generate(args.config)
    log(f"[rank {rank}] generated in {time.perf_counter() - t0:.1f}s: m_k={prob.m_k} "
        f"m_d={prob.m_d} n={prob.n} nnz_k={prob.meta['nnz_k']}")
    t0 = time.perf_counter()
    ctx = pkg.Context(prob, device=local)
    info = ctx.info()
    log(f"[rank {rank}] context in {time.perf_counter() - t0:.1f}s, "
        f"{info['device_bytes'] / 1e9:.1f} GB on device")
    bytes_it = info["hbm_bytes_iteration"]
    b = np.ascontiguousarray(prob.b_k)

    for _ in range(args.warmup):
        ctx.lsqr(b, lsqr_iteration=iters)
    if ws > 1:
        tdist.barrier()
    dev_s, wall = 0.0, 0.0
    with Clocks(local) as clk:
        for _ in range(args.steps):
            t = time.perf_counter()
            out = ctx.lsqr(b, lsqr_iteration=iters)  # host b in, host x out
            wall += time.perf_counter() - t
            dev_s += out["result"]["seconds"]
    dev_s, wall = max_over_ranks([dev_s, wall])
    clocks = clk.summary()
    value = ws * bytes_it * iters * args.steps / dev_s / 1e9
    e2e = ws * bytes_it * iters * args.steps / wall / 1e9

    # dominant kernel: time each product kernel alone (events on its stream)
    ms1 = ctx.bench_aprod(1, reps=10)
    ms2 = ctx.bench_aprod(2, reps=10)
    ms_it = ctx.bench_iteration(reps=20)
    dom_mode = 2 if ms2 >= ms1 else 1
    ms_dom = ms2 if dom_mode == 2 else ms1
    bytes_dom = info[f"hbm_bytes_aprod{dom_mode}"]
    peak, peak_kind = measured_peaks()
    achieved = bytes_dom / (ms_dom * 1e-3) / 1e9
    # the products as launched: the unit kernel over the slabs of the kernel
    # rows (mode 1) or columns (mode 2) and the kernel that adds the slab
    # partials with the damping part and the LSQR scaling
    kernels = {1: "aprod mode 1 (A x): k_slab_units<double> over K rows + k_combine_rows",
               2: "aprod mode 2 (A^T y): k_slab_units<double> over K columns + k_combine_cols"}
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": ncu_traffic(f"aprod_mode{dom_mode}"),
                "kernel": kernels[dom_mode], "peak_kind": peak_kind,
                "ms_per_launch": {"aprod_mode1": ms1, "aprod_mode2": ms2, "iteration": ms_it},
                "bytes_per_launch": bytes_dom}

    extra = {}
    if not args.no_tts and rank == 0:
        extra["time_to_1e-6"] = time_to_tol(pkg, prob, ctx, iters, 1e-6)
        if args.warm_train > 0:
            extra["warm_start"] = warm_time_to_tol(pkg, prob, ctx, iters, 1e-6, args.warm_train,
                                                   args.warm_epochs, args.warm_eval, local)
    ctx.close()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        orc = graft.load_oracle()
        s = cpu_sample(pkg, orc, prob, args.cpu_iterations)
        cpu = {"value": bytes_it * s["iterations"] / s["seconds"] / 1e9, "unit": UNIT,
               "cores": s["threads"], "kind": "port", "cpu_model": cpu_model(),
               "seconds_per_iteration": s["seconds"] / s["iterations"],
               "loop_seconds": s["seconds"],
               "wall_seconds_with_startup": s["wall_seconds"],
               "sample": cpu_sample_text(args.config, s["iterations"])
                         + f", {s['seconds']:.1f} s"}
    if rank != 0:
        return 0
    # per solve: start-up (sum of squares, norm, A^T y as unit product +
    # combine, update) and seven kernels per graph-replayed iteration (A x as
    # unit product + combine, norm, A^T y as unit product + combine, update,
    # tail); the ncu launch list of a 20-iteration solve counts 145
    launches = (5 + 7 * iters) * args.steps
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator, reference file formats)",
            "config": workload(args.config, prob, iters),
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 8 * prob.m_k,
                    "d2h_bytes_per_step": 8 * prob.n + 96 * (iters + 1) + 96},
            "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu,
            "clocks": clocks, **extra}
    print(json.dumps(line))
    return 0


def algorithmic_bytes(prob) -> float:
    """Bytes of one LSQR iteration, as plsqr_ctx_info computes them."""
    nk, nd = prob.meta["nnz_k"], prob.meta["nnz_d"]
    mk, md, n = prob.m_k, prob.m_d, prob.n
    a1 = 12.0 * (nk + nd) + 8.0 * (mk + 1 + md + 1) + 16.0 * (mk + md) + 8.0 * n
    a2 = 12.0 * (nk + nd) + 16.0 * (n + 1) + 16.0 * n + 8.0 * (mk + md)
    return a1 + a2 + 16.0 * (mk + md) + 8.0 * 6 * n


def workload(name, prob, iters) -> dict:
    return {"workload": f"{name}: FP64 LSQR, {iters} iterations, grid "
                        f"{'x'.join(map(str, prob.meta['grid']))}, {prob.m_k} rays "
                        f"(tube radius {prob.meta['tube_radius']})",
            "m_k": prob.m_k, "m_d": prob.m_d, "n": prob.n, "nnz_k": prob.meta["nnz_k"],
            "nnz_d": prob.meta["nnz_d"], "iterations": iters,
            "l2": "inputs larger than L2 (kernel matrix ~32 GB per iteration)"}


def time_to_tol(pkg, prob, ctx64, iters, tol) -> dict:
    """Device time to reach ||x - x*|| / ||x*|| <= tol, x* = the FP64 LSQR
    solution after twice the iteration count.  For each form a tracked run
    finds the first iteration below tol; then the same solve is run for
    exactly that many iterations, untracked, and timed from its first kernel
    to its last (start-up included; best of 3)."""
    xstar = ctx64.lsqr(lsqr_iteration=2 * iters)["x"]
    ctx64.set_reference_x(xstar)
    h = ctx64.lsqr(lsqr_iteration=2 * iters)["hist"]
    k64 = first_below(h["err"], tol)
    ctx64.set_reference_x(None)
    out = {"tol": tol, "reference": f"FP64 LSQR, {2 * iters} iterations"}
    if k64 is not None:
        t = [ctx64.lsqr(lsqr_iteration=k64)["result"]["seconds_total"] for _ in range(3)]
        out["fp64"] = {"iterations": k64, "seconds": min(t)}
    else:
        out["fp64"] = {"iterations": None, "final_err": float(h["err"][-1])}
    inner = 2 * iters
    with pkg.Context(prob, precision="mixed") as cm:
        cm.set_reference_x(xstar)
        hm = cm.lsqr(sweeps=2, inner=inner)["hist"]
        cm.set_reference_x(None)
        k = first_below(hm["err"], tol)
        if k is not None:
            sweeps = (k - 1) // inner + 1
            run = dict(sweeps=1, inner=k) if sweeps == 1 else dict(sweeps=sweeps, inner=inner)
            t = [cm.lsqr(**run)["result"]["seconds_total"] for _ in range(3)]
            out["mixed"] = {**run, "inner_iterations_to_tol": k, "seconds": min(t),
                            "form": "FP32 values (the hi half of the value split) times hi + lo "
                                    "FP32 pairs of the FP64 vectors, error-free FP32 products "
                                    "and sums, FP64 slab partials; FP64 vectors, norms and "
                                    "recurrence; FP64 residual refinement"}
            if "seconds" in out["fp64"]:
                out["speedup_mixed_vs_fp64"] = out["fp64"]["seconds"] / min(t)
        else:
            out["mixed"] = {"sweeps": None, "final_err": float(hm["err"][-1])}
        # the configuration's literal form: 50 inner iterations per sweep, up
        # to 6 sweeps; reported whether or not it reaches the tolerance
        cm.set_reference_x(xstar)
        hl = cm.lsqr(sweeps=6, inner=50)["hist"]
        cm.set_reference_x(None)
        kl = first_below(hl["err"], tol)
        lit = {"sweeps": 6, "inner": 50, "final_err": float(hl["err"][-1]),
               "inner_iterations_to_tol": kl,
               "seconds_6_sweeps": min(cm.lsqr(sweeps=6, inner=50)["result"]["seconds_total"]
                                       for _ in range(2))}
        if kl is not None:
            sw = (kl - 1) // 50 + 1
            lit["sweeps_to_tol"] = sw
            lit["seconds"] = min(cm.lsqr(sweeps=sw, inner=50)["result"]["seconds_total"]
                                 for _ in range(2))
        out["mixed_50_per_sweep"] = lit
        if "seconds" in out.get("mixed", {}):
            ms = cm.bench_iteration(reps=20)
            out["mixed"]["ms_per_inner_iteration"] = ms
    # FP32 vectors in the inner sweeps as well (PLSQR_MIXED_F32VEC=1)
    os.environ["PLSQR_MIXED_F32VEC"] = "1"
    try:
        with pkg.Context(prob, precision="mixed") as cf:
            cf.set_reference_x(xstar)
            hf = cf.lsqr(sweeps=2, inner=inner)["hist"]
            cf.set_reference_x(None)
            k = first_below(hf["err"], tol)
            row = {"form": "FP32 products and FP32 vectors in the inner sweeps; FP64 norms, "
                           "recurrence and residual refinement", "final_err": float(hf["err"][-1]),
                   "inner_iterations_to_tol": k, "ms_per_inner_iteration": cf.bench_iteration(reps=20)}
            if k is not None:
                sweeps = (k - 1) // inner + 1
                run = dict(sweeps=1, inner=k) if sweeps == 1 else dict(sweeps=sweeps, inner=inner)
                row["seconds"] = min(cf.lsqr(**run)["result"]["seconds_total"] for _ in range(3))
                row.update(run)
            out["mixed_f32_vectors"] = row
    finally:
        os.environ.pop("PLSQR_MIXED_F32VEC", None)
    out["fp64"]["ms_per_iteration"] = ctx64.bench_iteration(reps=20)
    return out


def warm_time_to_tol(pkg, prob, ctx64, iters, tol, n_train, epochs, n_eval, device) -> dict:
    """The target form: learned warm start + mixed precision, against
    plain FP64 LSQR and cold mixed precision, time to `tol` relative error vs
    each instance's FP64 solution (FP64 LSQR run to twice the iterations).

    A bounded version of `--extension warm`: the U-Net is trained here on
    n_train (A^T b, x_LSQR) pairs of the model class (the batched mixed solver
    makes x_LSQR), for `epochs` passes, and evaluated on n_eval held-out
    instances of the same class.  The warm time includes the back-projection
    and the network."""
    W = pkg.warm
    grid = prob.meta["grid"]
    t0 = time.perf_counter()
    cn2 = W.column_norms2(prob)

    def instance(seed):
        x_true, b = W.measurements(ctx64, "grid96", grid, seed)
        return b, W.back_projection(ctx64, b, cn2).astype(np.float32)

    tr = [instance(s) for s in range(n_train)]
    x_tr, _, _ = W.solve_batches(ctx64, [b for b, _ in tr], iters)
    t_data = time.perf_counter() - t0
    rms = lambda v: float(np.sqrt(np.mean(np.asarray(v, np.float64) ** 2)))
    c = float(np.median([rms(x) / max(rms(z), 1e-300) for x, (_, z) in zip(x_tr, tr)]))
    t0 = time.perf_counter()
    net = W.UNet(grid, seed=1, device=device)
    total, step = epochs * n_train, 0
    for ep in range(epochs):
        for i in np.random.default_rng(ep).permutation(n_train):
            lr = 1e-5 + 0.5 * (1e-3 - 1e-5) * (1.0 + np.cos(np.pi * step / total))
            net.train_step(tr[i][1], (x_tr[i] / c).astype(np.float32), lr)
            step += 1
    t_train = time.perf_counter() - t0
    rows = []
    with pkg.Context(prob, precision="mixed", device=device) as cm:
        for j in range(n_eval):
            b, z = instance(1_000_000 + j)
            xs = ctx64.lsqr(b, lsqr_iteration=2 * iters)["x"]
            ctx64.set_reference_x(xs)
            k64 = first_below(ctx64.lsqr(b, lsqr_iteration=2 * iters)["hist"]["err"], tol)
            ctx64.set_reference_x(None)
            cm.set_reference_x(xs)
            kc = first_below(cm.lsqr(b, sweeps=1, inner=2 * iters)["hist"]["err"], tol)
            tp = time.perf_counter()
            x0 = c * net.predict(W.back_projection(ctx64, b, cn2))
            t_pre = time.perf_counter() - tp
            hw = cm.lsqr(b, sweeps=1, inner=2 * iters, x0=x0)
            kw = first_below(hw["hist"]["err"], tol)
            cm.set_reference_x(None)
            row = {"x0_rel_err": float(np.linalg.norm(x0 - xs) / np.linalg.norm(xs)),
                   "kept_x0": int(hw["result"]["warm"])}
            if k64 is not None:
                row["fp64"] = {"iterations": k64, "seconds": min(
                    ctx64.lsqr(b, lsqr_iteration=k64)["result"]["seconds_total"] for _ in range(2))}
            if kc is not None:
                row["mixed"] = {"iterations": kc, "seconds": min(
                    cm.lsqr(b, sweeps=1, inner=kc)["result"]["seconds_total"] for _ in range(2))}
            if kw is not None:
                row["warm_mixed"] = {"iterations": kw, "x0_seconds": t_pre, "seconds": t_pre + min(
                    cm.lsqr(b, sweeps=1, inner=kw, x0=x0)["result"]["seconds_total"]
                    for _ in range(2))}
            rows.append(row)
    net.close()
    out = {"tol": tol, "train_pairs": n_train, "epochs": epochs, "heldout_instances": n_eval,
           "data_seconds": t_data, "train_seconds": t_train, "instances": rows,
           "model_class": "16-128 Gaussian blobs + checkerboard of period 4-16, 1% noise, "
                          "measured through the benchmark's kernel matrix",
           "target": "warm start + mixed precision >= 3x faster than plain FP64"}
    ok = [r for r in rows if all(k in r for k in ("fp64", "mixed", "warm_mixed"))]
    if ok:
        t = {k: float(np.mean([r[k]["seconds"] for r in ok])) for k in ("fp64", "mixed", "warm_mixed")}
        out["mean_seconds"] = t
        out["speedup_mixed_vs_fp64"] = t["fp64"] / t["mixed"]
        out["speedup_warm_mixed_vs_fp64"] = t["fp64"] / t["warm_mixed"]
    return out


# ---- extensions ---------------------------------------------------------------------
def bench_batched(pkg, args, device) -> dict:
    """32 right-hand sides on the 96x96x32 operator (16 noise seeds, 8 damping
    weights, 8 checkerboards): time until every one is within 1e-6 of its own
    FP64 solution, batched against the plain FP64 path run once per
    right-hand side.  Batched two ways: all 32 in lock step until the slowest
    is done, and grouped by iterations to the tolerance (a batch per group,
    the block width shrinking with the group)."""
    tol = 1e-6
    name = args.config
    iters = args.iterations or pkg.CONFIGS[name]["iterations"]
    prob = pkg.generate(name)
    ctx = pkg.Context(prob, device=device)
    insts = pkg.batch.instances(ctx, prob, name)
    ms_it = None
    per = []
    xstar = []
    long_iters = 6 * iters
    for inst in insts:
        ctx.set_damping_weight(inst.lam)
        # reference solution: FP64 LSQR over twice the iterations, or six
        # times where the tolerance comes only near the end of that run (the
        # smallest damping weights converge slowly)
        for ref_it in (2 * iters, long_iters):
            xs = ctx.lsqr(inst.b_k, lsqr_iteration=ref_it)["x"]
            ctx.set_reference_x(xs)
            h = ctx.lsqr(inst.b_k, lsqr_iteration=ref_it)["hist"]
            ctx.set_reference_x(None)
            k = first_below(h["err"], tol)
            if k is not None and k < 0.95 * ref_it:
                break
        if ms_it is None:
            ms_it = ctx.bench_iteration(reps=20)
        per.append({"name": inst.name, "lambda": inst.lam, "fp64_iterations": k,
                    "reference_iterations": ref_it})
        xstar.append(xs)
        log(f"{inst.name}: FP64 reaches {tol:g} at {k} (reference {ref_it} iterations)")
    ctx.set_damping_weight(1.0)
    # plain FP64, one solve per right-hand side: iterations x graph-replayed
    # iteration time, plus the start-up (a plain solve of 0 iterations)
    t0 = ctx.lsqr(insts[0].b_k, lsqr_iteration=1)["result"]
    startup = max(t0["seconds_total"] - t0["seconds"], 0.0)
    b = np.stack([i.b_k for i in insts])
    lam = [i.lam for i in insts]
    X = np.stack(xstar)
    # tracked run: one sweep long enough for the slowest instance
    inner = 2 * max(p["reference_iterations"] for p in per)
    tr = ctx.batch_lsqr(b, lam=lam, x_ref=X, sweeps=1, inner=inner)
    ks = [first_below(tr["hist"]["err"][j], tol) for j in range(len(insts))]
    for p, k, h in zip(per, ks, tr["hist"]["err"]):
        p["batched_iterations"] = k
        p["batched_final_err"] = float(h[-1])
    # instances whose FP64 path only reaches the tolerance near the end of
    # even the long reference run have no converged reference solution:
    # reported, not timed
    ok = [p["fp64_iterations"] is not None and p["fp64_iterations"] < 0.95 * p["reference_iterations"]
          for p in per]
    for p, o in zip(per, ok):
        p["timed"] = bool(o)
    out = {"metric": "time to 1e-6 rel. error for 32 right-hand sides (vs each one's FP64 "
                     "solution)", "unit": "s", "higher_is_better": False,
           "extension": "batched", "n_gpus": 1, "dtype": "f32 products / f64 vectors",
           "data": "synthetic (seeded generator)",
           "config": {"workload": f"{name}: 32 right-hand sides (16 noise seeds, 8 damping "
                                  f"weights 0.1-10, 8 checkerboards period 4-16)",
                      "m_k": prob.m_k, "n": prob.n, "nnz_k": prob.meta["nnz_k"],
                      "reference_solutions": f"FP64 LSQR, {2 * iters} iterations each "
                                             f"({long_iters} where that does not converge)"},
           "instances": per, "variants": tr["info"]}
    timed = [j for j, o in enumerate(ok) if o]
    if all(ks[j] is not None for j in timed):
        fp64_total = sum(startup + per[j]["fp64_iterations"] * ms_it * 1e-3 for j in timed)
        # (a) lock step: all 32 until the slowest timed instance is within tol
        K = max(ks[j] for j in timed)
        lock = min(ctx.batch_lsqr(b, lam=lam, sweeps=1, inner=K)["results"][0]["seconds"]
                   for _ in range(2))
        # (b) grouped by iterations to tol: the timed instances sorted by their
        # count and cut into consecutive groups, each run as its own batch to
        # its slowest member, or (a group of one) on the one-right-hand-side
        # mixed solver; the cut minimises the modelled time (measured
        # iteration time of each block width, or of the mixed solver, x the
        # group's count)
        order = sorted(timed, key=lambda j: ks[j])
        it_ms = {}
        for kw in (4, 8, 16, 32):
            it_ms[kw] = (ctx.batch_bench_aprod(kw, 1, reps=3) + ctx.batch_bench_aprod(kw, 2, reps=3))
        cm = pkg.Context(prob, device=device, precision="mixed")
        cm.set_damping_weight(lam[order[0]])
        cm.lsqr(prob.b_k, sweeps=1, inner=5)
        mixed_ms = cm.bench_iteration(reps=20)
        width = lambda c: 4 if c <= 4 else 8 if c <= 8 else 16 if c <= 16 else 32
        nt = len(order)
        best = [0.0] + [float("inf")] * nt
        cut = [0] * (nt + 1)
        for e in range(1, nt + 1):
            for s0 in range(e):
                c = best[s0] + min(it_ms[width(e - s0)],
                                   mixed_ms if e - s0 == 1 else float("inf")) * ks[order[e - 1]]
                if c < best[e]:
                    best[e], cut[e] = c, s0
        groups, e = [], nt
        while e > 0:
            groups.append(order[cut[e]:e])
            e = cut[e]
        groups.reverse()
        grouped = 0.0
        ginfo = []
        for gidx in groups:
            kg = max(ks[j] for j in gidx)
            tb = None
            if len(gidx) > 1 or it_ms[4] <= mixed_ms:
                tb = min(ctx.batch_lsqr(b[gidx], lam=[lam[j] for j in gidx], sweeps=1,
                                        inner=kg)["results"][0]["seconds"] for _ in range(2))
                ginfo.append({"instances": [per[j]["name"] for j in gidx], "iterations": kg,
                              "solver": f"batched, block width {width(len(gidx))}",
                              "seconds": tb})
                grouped += tb
                continue
            j = gidx[0]  # one right-hand side: the mixed solver, its own count
            cm.set_damping_weight(lam[j])
            cm.set_reference_x(X[j])
            km = first_below(cm.lsqr(b[j], sweeps=1, inner=2 * kg)["hist"]["err"], tol)
            cm.set_reference_x(None)
            if km is None:  # not within tol on the mixed solver: the batch instead
                tb = min(ctx.batch_lsqr(b[gidx], lam=[lam[j]], sweeps=1, inner=kg)
                         ["results"][0]["seconds"] for _ in range(2))
                ginfo.append({"instances": [per[j]["name"]], "iterations": kg,
                              "solver": "batched, block width 4", "seconds": tb})
                grouped += tb
                continue
            tm = min(cm.lsqr(b[j], sweeps=1, inner=km)["result"]["seconds_total"]
                     for _ in range(2))
            ginfo.append({"instances": [per[j]["name"]], "iterations": km,
                          "solver": "mixed precision, one right-hand side", "seconds": tm})
            grouped += tm
        cm.close()
        # (c) retirement: the timed instances in one batch, each leaving as it
        # comes within tol (checked every 16 iterations), the rest packed into
        # the narrowest block that holds them; no counts known in advance
        tb = b[timed]
        rts = [ctx.batch_lsqr(tb, lam=[lam[j] for j in timed], x_ref=X[timed], sweeps=1,
                              inner=inner, retire_every=16, retire_err=tol) for _ in range(2)]
        rt = min(rts, key=lambda r: r["results"][0]["seconds"])
        rt_err = [float(np.linalg.norm(rt["x"][i] - X[j]) / np.linalg.norm(X[j]))
                  for i, j in enumerate(timed)]
        retire = {"seconds": rt["results"][0]["seconds"], "check_every": 16,
                  "iterations": {per[j]["name"]: rt["results"][i]["itn"]
                                 for i, j in enumerate(timed)},
                  "max_error": max(rt_err),
                  "speedup_vs_fp64_sequential": fp64_total / rt["results"][0]["seconds"]}
        out.update(value=grouped, timed_instances=len(timed), retire=retire,
                   fp64_sequential_seconds=fp64_total,
                   speedup_vs_fp64_sequential=fp64_total / grouped,
                   lock_step={"seconds": lock, "iterations": K,
                              "speedup_vs_fp64_sequential": fp64_total / lock},
                   groups=ginfo, iteration_ms_by_width=it_ms, mixed_iteration_ms=mixed_ms,
                   note="value: the timed instances grouped by their iterations to the "
                        "tolerance, each group run as one batch (one sweep, to its slowest "
                        "member) or, a group of one, on the mixed-precision solver; device "
                        "time summed; lock_step: all 32 right-hand sides in one batch until "
                        "the slowest timed one is within the tolerance; retire: the timed "
                        "ones in one batch, each retiring as it comes within the tolerance "
                        "and the rest packed into narrower blocks; "
                        "fp64_sequential_seconds: the timed instances one after another on "
                        "the plain FP64 path")
    else:
        out.update(value=None, note="not every right-hand side reached the tolerance")
    ms1 = ctx.batch_bench_aprod(32, 1, reps=3)
    ms2 = ctx.batch_bench_aprod(32, 2, reps=3)
    nk = prob.meta["nnz_k"]
    out["products"] = {"ms_ax": ms1, "ms_aty": ms2, "fp64_iteration_ms": ms_it,
                       "gather_bytes_per_product": 128.0 * nk,
                       "gather_tb_s": {"ax": 128.0 * nk / ms1 / 1e9, "aty": 128.0 * nk / ms2 / 1e9},
                       "matrix_gb_s": {"ax": 8.0 * nk / ms1 / 1e6, "aty": 8.0 * nk / ms2 / 1e6}}
    ctx.close()
    return out


def bench_uneven(pkg, args, device) -> dict:
    """The 24 uneven problems (16^3-64^3 grids, 500-20,000 rays, 100 FP64 LSQR
    iterations each): one persistent launch against one plain solve per
    problem (each with its own graph-replayed iterations) on the same GPU."""
    probs = [pkg.generate(c) for c in pkg.multi.uneven_configs()]
    with pkg.multi.Multi(probs, device=device) as mp:
        for _ in range(max(args.warmup, 1)):
            mp.solve()
        t = []
        for _ in range(max(args.steps, 1)):
            out = mp.solve()
            t.append(out["seconds"])
        info = mp.info()
        g, gb = mp.plan()
        # the configuration's form: FP32 inner / FP64 outer, the same
        # iteration count per sweep
        mixed = {}
        for sw in (2, 3):
            mp.set_mixed(sw)
            mp.solve()
            tm = [mp.solve() for _ in range(max(args.steps, 1))]
            mixed[sw] = (min(r["seconds"] for r in tm), tm[0]["x"])
        mp.set_mixed(0)
    seq, worst = 0.0, 0.0
    err64, errm = [], {sw: [] for sw in mixed}
    for i, (p, x) in enumerate(zip(probs, out["x"])):
        with pkg.Context(p, device=device) as c:
            c.lsqr(lsqr_iteration=p.iterations)
            r = min((c.lsqr(lsqr_iteration=p.iterations) for _ in range(2)),
                    key=lambda r: r["result"]["seconds_total"])
            xs = c.lsqr(lsqr_iteration=8 * p.iterations)["x"]  # converged FP64 solution
        seq += r["result"]["seconds_total"]
        worst = max(worst, float(np.linalg.norm(x - r["x"]) / np.linalg.norm(r["x"])))
        nx = np.linalg.norm(xs)
        err64.append(float(np.linalg.norm(x - xs) / nx))
        for sw in mixed:
            errm[sw].append(float(np.linalg.norm(mixed[sw][1][i] - xs) / nx))
    its = sum(p.iterations for p in probs)
    return {"metric": "24 uneven FP64 LSQR problems (100 iterations each) in one persistent "
                      "launch: device time", "unit": "s", "value": min(t),
            "higher_is_better": False, "extension": "uneven", "n_gpus": 1, "dtype": "f64",
            "data": "synthetic (seeded generator)",
            "config": {"workload": "24 problems: grids 16^3-64^3, 500-20000 rays, tube radius "
                                   "1.5", "nnz_k": [p.meta["nnz_k"] for p in probs],
                       "blocks": info["blocks"], "blocks_per_problem": gb[g].tolist()},
            "sequential_seconds": seq, "speedup_vs_sequential": seq / min(t),
            "problem_iterations_per_s": its / min(t),
            "max_rel_diff_vs_one_problem_path": worst,
            "rel_err_vs_converged_fp64": {
                "reference": "FP64 LSQR of each problem, 8x its iteration count",
                "fp64_one_lsqr": err64,
                **{f"mixed_{sw}_sweeps": errm[sw] for sw in mixed}},
            "mixed": {f"{sw}_sweeps": {"seconds": mixed[sw][0],
                                       "max_rel_err": max(errm[sw]),
                                       "median_rel_err": float(np.median(errm[sw]))}
                      for sw in mixed},
            "mixed_form": "FP32 inner / FP64 outer: sweeps of the problem's iteration count "
                          "on the FP64 residual, FP32 kernel values times hi + lo FP32 pairs "
                          "of the FP64 vectors (error-free FP32 products and sums)"}


def bench_warm(pkg, args, device) -> dict:
    """Learned warm start on the 96x96x32 geometry: train the U-Net on
    (column-norm-scaled A^T b, x_LSQR) pairs of seeded models, then compare,
    on held-out seeds, the iterations and time to 1e-6 of each one's FP64
    solution for plain FP64 LSQR (cold), mixed precision (cold) and mixed
    precision from the network's x0 (warm, cold start as fallback)."""
    tol = 1e-6
    name = args.config
    iters = args.iterations or pkg.CONFIGS[name]["iterations"]
    W = pkg.warm
    t_all = time.perf_counter()
    prob = pkg.generate(name)
    grid = prob.meta["grid"]
    ctx = pkg.Context(prob, device=device)
    cn2 = W.column_norms2(prob)
    seeds_train = list(range(args.train))
    seeds_test = list(range(1_000_000, 1_000_000 + args.heldout))

    def inputs(seeds):
        zs, bs, xt = [], [], []
        for s in seeds:
            x_true, b = W.measurements(ctx, name, grid, s)
            bs.append(b)
            xt.append(x_true)
            zs.append(W.back_projection(ctx, b, cn2).astype(np.float32))
        return zs, bs, xt

    t0 = time.perf_counter()
    z_tr, b_tr, _ = inputs(seeds_train)
    x_tr, _, _ = W.solve_batches(ctx, b_tr, iters)
    x_tr = [x.astype(np.float32) for x in x_tr]
    del b_tr
    t_data = time.perf_counter() - t0
    log(f"training pairs: {len(x_tr)} in {t_data:.1f}s")
    # one global factor brings the solutions to the inputs' scale (the
    # network itself divides its input by, and multiplies its output with,
    # the input's root mean square)
    rms = lambda v: float(np.sqrt(np.mean(v * v)))
    c = float(np.median([rms(x.astype(np.float64)) / max(rms(z.astype(np.float64)), 1e-300)
                         for x, z in zip(x_tr, z_tr)]))
    z_te, b_te, _ = inputs(seeds_test)
    x_te, _, _ = W.solve_batches(ctx, b_te, iters)

    def rel_err(net, js):
        return [float(np.linalg.norm(c * net.predict(z_te[j]) - x_te[j]) / np.linalg.norm(x_te[j]))
                for j in js]

    losses, curve = [], []
    t0 = time.perf_counter()
    net = W.UNet(grid, seed=1, device=device)
    total, step = args.epochs * len(z_tr), 0
    for ep in range(args.epochs):
        order = np.random.default_rng(ep).permutation(len(z_tr))
        for i in order:
            # cosine decay of the step size from 1e-3 to 1e-5
            lr = 1e-5 + 0.5 * (1e-3 - 1e-5) * (1.0 + np.cos(np.pi * step / total))
            losses.append(net.train_step(z_tr[i], x_tr[i] / c, lr))
            step += 1
        e = float(np.median(rel_err(net, range(min(32, len(z_te))))))
        curve.append({"epoch": ep, "loss": float(np.mean(losses[-len(order):])),
                      "heldout_rel_err": e})
        log(f"epoch {ep}: mean loss {curve[-1]['loss']:.4f}, held-out x0 error {e:.4f}")
    t_train = time.perf_counter() - t0
    x0_te = [c * net.predict(z) for z in z_te]
    pred_err = [float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(x0_te, x_te)]
    # timed subset: FP64 reference solutions (twice the iterations), then cold
    # and warm tracked runs
    nt = min(args.timed, len(seeds_test))
    xstar, k64 = [], []
    for j in range(nt):
        xs = ctx.lsqr(b_te[j], lsqr_iteration=2 * iters)["x"]
        ctx.set_reference_x(xs)
        h = ctx.lsqr(b_te[j], lsqr_iteration=2 * iters)["hist"]
        ctx.set_reference_x(None)
        xstar.append(xs)
        k64.append(first_below(h["err"], tol))
    ms_fp64 = ctx.bench_iteration(reps=20)
    inner = 2 * iters
    _, h_cold, s_cold = W.solve_batches(ctx, b_te[:nt], inner, x_refs=xstar)
    _, h_warm, s_warm = W.solve_batches(ctx, b_te[:nt], inner, x0s=x0_te[:nt], x_refs=xstar)
    k_cold = [first_below(h["err"], tol) for h in h_cold]
    k_warm = [first_below(h["err"], tol) for h in h_warm]
    # how the savings grow with the accuracy of x0: the network's error
    # scaled down by 10 and 100 (x0 = x* + t (x0_net - x*))
    scaled = {}
    if nt:
        ts = (0.1, 0.01)
        x0s = [xstar[j] + t * (x0_te[j] - xstar[j]) for t in ts for j in range(nt)]
        _, h_sc, _ = W.solve_batches(ctx, b_te[:nt] * len(ts), inner, x0s=x0s,
                                     x_refs=xstar * len(ts))
        k_sc = [first_below(h["err"], tol) for h in h_sc]
        for i, t in enumerate(ts):
            ks = [k for k in k_sc[i * nt:(i + 1) * nt] if k is not None]
            scaled[f"error_x{t:g}"] = float(np.mean(ks)) if ks else None
    # one right-hand side at a time, as a user solves: device time to 1e-6
    # of FP64 LSQR, of the mixed solve, and of back-projection + network +
    # mixed solve from x0 (host wall time of the first two, with their copies)
    single = []
    with pkg.Context(prob, precision="mixed", device=device) as cm:
        for j in range(min(args.timed_single, nt)):
            if k64[j] is None:
                continue
            row = {"fp64": {"iterations": k64[j], "seconds": min(
                ctx.lsqr(b_te[j], lsqr_iteration=k64[j])["result"]["seconds_total"]
                for _ in range(2))}}
            cm.set_reference_x(xstar[j])
            kc = first_below(cm.lsqr(b_te[j], sweeps=1, inner=inner)["hist"]["err"], tol)
            t0 = time.perf_counter()
            x0 = c * net.predict(W.back_projection(ctx, b_te[j], cn2))
            t_pre = time.perf_counter() - t0
            hw = cm.lsqr(b_te[j], sweeps=1, inner=inner, x0=x0)
            kw = first_below(hw["hist"]["err"], tol)
            cm.set_reference_x(None)
            if kc is None or kw is None:
                continue
            row["mixed"] = {"iterations": kc, "seconds": min(
                cm.lsqr(b_te[j], sweeps=1, inner=kc)["result"]["seconds_total"]
                for _ in range(2))}
            row["mixed_warm"] = {"iterations": kw, "kept_x0": hw["result"]["warm"],
                                 "x0_seconds": t_pre, "seconds": t_pre + min(
                cm.lsqr(b_te[j], sweeps=1, inner=kw, x0=x0)["result"]["seconds_total"]
                for _ in range(2))}
            single.append(row)
    net.close()
    ok = [a is not None and b is not None and c is not None for a, b, c in zip(k64, k_cold, k_warm)]
    sel = [j for j in range(nt) if ok[j]]
    out = {"metric": "iterations to 1e-6 rel. error (vs FP64 solution), held-out seeds: "
                     "FP64 cold / mixed cold / mixed from the learned warm start",
           "unit": "iterations", "extension": "warm", "higher_is_better": False, "n_gpus": 1,
           "dtype": "bf16 network, f32 products / f64 vectors",
           "data": "synthetic (seeded models: 16-128 blobs + checkerboard, 1% noise)",
           "config": {"workload": f"{name} geometry, U-Net 16/32/64 channels",
                      "train_pairs": len(x_tr), "epochs": args.epochs,
                      "heldout": len(seeds_test), "timed": nt},
           "train_seconds": t_train, "data_seconds": t_data, "target_scale": c,
           "training_curve": curve,
           "x0_rel_err_vs_x_lsqr": {"median": float(np.median(pred_err)),
                                    "p90": float(np.percentile(pred_err, 90))},
           "per_instance": [{"fp64": k64[j], "mixed_cold": k_cold[j], "mixed_warm": k_warm[j]}
                            for j in range(nt)],
           "fp64_iteration_ms": ms_fp64,
           "iterations_with_x0_error_scaled": scaled,
           "single_rhs": single,
           "seconds_total": time.perf_counter() - t_all}
    if sel:
        m64 = float(np.mean([k64[j] for j in sel]))
        mc = float(np.mean([k_cold[j] for j in sel]))
        mw = float(np.mean([k_warm[j] for j in sel]))
        out.update(value=mw, mean_iterations={"fp64": m64, "mixed_cold": mc, "mixed_warm": mw},
                   warm_over_cold_iterations=mc / mw)
    if single:
        t64 = float(np.mean([r["fp64"]["seconds"] for r in single]))
        out["time_to_1e-6_single_rhs"] = {
            "instances": len(single), "fp64_s": t64,
            "mixed_s": float(np.mean([r["mixed"]["seconds"] for r in single])),
            "warm_mixed_s": float(np.mean([r["mixed_warm"]["seconds"] for r in single]))}
        out["time_to_1e-6_single_rhs"]["speedup_warm_mixed_vs_fp64"] = \
            t64 / out["time_to_1e-6_single_rhs"]["warm_mixed_s"]
    ctx.close()
    return out


if __name__ == "__main__":
    sys.exit(main())

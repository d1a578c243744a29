#!/usr/bin/env python
"""Throughput benchmark of the GB300 line-intensity engine.

Workload (default ``c2v_plain``): triatomic C2v, J = 0..10, Nvib = 2000,
the lowest 1000 eigenvectors per (J, Gamma) under 15000 cm^-1, every
dJ = 0, +-1 block pair; seeded synthetic inputs of those shapes (no TROVE
checkpoints exist here).  One step = one whole intensity job over that
input: every line S, A_if, I(T) after the reference's filters.

Metric: linestrengths/s, counting lines that pass every filter before the
intensity threshold (1e-30 cm/molecule; the post-threshold count is reported
beside it).

  value   inputs resident in HBM, lines kept on the device, CUDA-event time
          of K steps on the engine's stream, bracketed by synchronize (and a
          barrier across ranks); each step is one CUDA-graph launch
  e2e     the same job through the C ABI from pinned host buffers: every step
          uploads the dipole and every eigenvector block and reads all lines
          back to host memory
  roofline    the half-ls split GEMM's algorithmic TFLOP/s against the
          measured bf16 peak, with its DRAM traffic
  fp64_path / accuracy   the FP64 GPU path on the same job; split vs FP64
          error per line on its J <= 3 part
  serving     pair jobs arriving as a Poisson stream through gi_serve_*
  dipole_streamed   the job with its dipole kept in host memory and streamed
          in four panels
  cpu_baseline / --impl reference   the reference's algorithm on the host
          cores (the CPU oracle port; the reference has no CPU implementation
          of the path) on a bounded sample of the same workload

Multi-GPU (torchrun): every rank runs an independent replica of the job with
its own seed (no collective on the data path), value = all ranks' lines /
max time ("weak" scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as G  # noqa: E402

METRIC = "linestrengths/s"
THRESH_I = 1e-30  # cm/molecule
# DRAM bytes (read + write) of one half-line-strength k_split_gemm_g launch per Y
# column: ncu on the J <= 4 part of c2v_plain measured 62.14 GB + 6.54 GB for a
# launch of 1000 x 96-column tiles.
SPLIT_HALFLS_DRAM_BYTES_PER_COL = (62.136866e9 + 6.543222e9) / 96000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2v_plain")
    ap.add_argument("--jmax", type=int, default=None, help="restrict J to 0..jmax")
    ap.add_argument("--precision", default="split", choices=["fp64", "split"])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--slices", type=int, default=0, help="bf16 digits per operand (split)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64-path comparison")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-stream", action="store_true",
                    help="skip the streamed-dipole measurement")
    ap.add_argument("--serve-jmax", type=int, default=4,
                    help="serving: pair jobs of the J <= jmax part of the workload")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="serving: Poisson jobs/s")
    ap.add_argument("--serve-slots", type=int, default=3)
    ap.add_argument("--tune-table", default=None,
                    help="autotuner table file: read if present, extended and written")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def across_ranks(dt, lines_pre, lines_post, device):
    """Every rank times its own replica of the job: the whole job's step time is
    the slowest rank's and its lines are all ranks' lines (one process: as is)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return dt, lines_pre, lines_post
    t = torch.tensor([dt], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([float(lines_pre), float(lines_post)], dtype=torch.float64, device=device)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(t.item()), int(n[0].item()), int(n[1].item())


def make_problem(args, rank=0):
    G.load_package()
    from gpu_intensities_gb300 import synth
    kw = {}
    if args.jmax is not None:
        kw["jlist"] = list(range(args.jmax + 1))
    prob = synth.workload(args.workload, seed=args.seed + rank, **kw)
    prob.params.thresh_intensity = THRESH_I
    return prob


def config_of(args, prob):
    return {"workload": args.workload, "sym": "C2v" if prob.sym_type == 1 else "C3v",
            "J": [min(prob.jlist), max(prob.jlist)], "Nvib": prob.N,
            "nvec_max_per_block": max(b.nvec for b in prob.blocks.values()),
            "levels": int(sum(b.nvec for b in prob.blocks.values())),
            "precision": args.precision, "thresh_intensity_cm_per_molecule": THRESH_I,
            "l2": "inputs (eigenvector blocks, 1.9 GB) larger than L2",
            "seed": args.seed}


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock and throttle-reason samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.index)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        rows = []
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), float(f[3]) if f[3] not in ("[N/A]",) else 0.0,
                             f[5], f[6], f[7], f[8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [r[0] for r in rows]
        reasons = []
        for i, name in ((3, "hw_slowdown"), (4, "hw_thermal_slowdown"),
                        (5, "sw_thermal_slowdown"), (6, "sw_power_cap")):
            if any(r[i].lower() == "active" for r in rows):
                reasons.append(name)
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------- CPU baseline
def cpu_sample(prob, nlow: int):
    """Bounded sample of the workload for the oracle: the reference run over the
    two highest J with only the nlow lowest initial levels kept (lower energy
    window), every final level kept."""
    O = G.load_oracle()
    js = prob.jlist
    pair = (js[-2], js[-1])
    zpe = O.resolve_zpe(prob)
    e = np.sort(np.concatenate([prob.blocks[(J, g)].energies for J in pair
                                for g in range(prob.nrep) if (J, g) in prob.blocks]))
    cut = float(e[min(nlow, len(e)) - 1]) - (zpe if zpe > 0 else 0.0)
    saved = prob.params.erange_lower
    prob.params.erange_lower = (saved[0], cut)
    return O, pair, zpe, saved


def run_cpu(prob, nlow: int, threads: int):
    O, pair, zpe, saved = cpu_sample(prob, nlow)
    try:
        t = time.perf_counter()
        lines = O.run_pair(prob, pair, zpe, nthreads=threads)
        dt = time.perf_counter() - t
    finally:
        prob.params.erange_lower = saved
    return len(lines), dt, pair


def cpu_baseline(prob, nlow=8):
    threads = os.cpu_count() or 1
    n, dt, pair = run_cpu(prob, nlow, threads)
    return {"value": n / dt, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"oracle run over J={pair[0]},{pair[1]} restricted to the {nlow} lowest "
                      f"initial levels ({n} lines in {dt:.1f} s)"}


# ---------------------------------------------------------------- accuracy
def split_accuracy(pkg, prob, slices, device):
    """Split path against the FP64 GPU path (itself parity-tested against the
    CPU oracle) on the J <= 3 part of the workload: identical line selection
    and the per-line relative error of S."""
    from gpu_intensities_gb300 import synth
    sub = synth.Problem(prob.sym_type, prob.N, prob.mu,
                        {J: b for J, b in prob.bases.items() if J <= 3},
                        {k: b for k, b in prob.blocks.items() if k[0] <= 3}, prob.params,
                        name=prob.name + "_J0-3")
    out = {}
    for name, prec in (("fp64", pkg.GI_PREC_FP64), ("split", pkg.GI_PREC_SPLIT)):
        with pkg.Engine(device) as e:
            e.load(sub, precision=prec, split_slices=slices)
            e.run()
            out[name] = pkg.keyed(e.lines(), e.levels())
    a, b = out["fp64"], out["split"]
    keys = ("jI", "gammaI", "recI", "jF", "gammaF", "recF")
    a = a[np.lexsort(tuple(a[k] for k in reversed(keys)))]
    b = b[np.lexsort(tuple(b[k] for k in reversed(keys)))]
    same = len(a) == len(b) and all(np.array_equal(a[k], b[k]) for k in keys)
    res = {"sample": "J<=3 part of the workload, split vs FP64 GPU path",
           "lines": int(len(a)), "identical_selection": bool(same)}
    if same and len(a):
        rel = np.abs(b["S"] - a["S"]) / np.where(a["S"] > 0, a["S"], 1.0)
        tmax = np.abs(a["t"]).max()
        well = np.abs(a["t"]).max(axis=1) >= 1e-4 * tmax
        res.update({"rel_err_S_max": float(rel.max()), "rel_err_S_p99": float(np.quantile(rel, 0.99)),
                    "rel_err_S_max_well_conditioned": float(rel[well].max()),
                    "well_conditioned_fraction": float(well.mean()),
                    "note": "well conditioned: |t| >= 1e-4 max|t| (no cancellation beyond 1e4)"})
    return res


# ---------------------------------------------------------------- reference arm
def main_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    prob = make_problem(args)
    threads = os.cpu_count() or 1
    nlow = 4
    for _ in range(args.warmup):
        run_cpu(prob, nlow, threads)
    tot_n, tot_t = 0, 0.0
    for _ in range(args.steps):
        n, dt, pair = run_cpu(prob, nlow, threads)
        tot_n += n
        tot_t += dt
    v = tot_n / tot_t
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC,
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": config_of(args, prob),
           "cpu_baseline": {"value": v, "unit": METRIC, "cores": threads, "kind": "port",
                            "sample": f"oracle (the reference's algorithm restated in C; the "
                                      f"reference has no CPU path) over J={pair[0]},{pair[1]} "
                                      f"with the {nlow} lowest initial levels per step"},
           "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


# ---------------------------------------------------------------- serving
def serve_bench(pkg, args, device, precision):
    """Pair jobs (J, Gamma) -> (J', Gamma') of the J <= serve_jmax part of the
    workload, submitted in random order with Poisson arrivals at serve_rate
    jobs/s to a serving context; latency is submit -> lines on the host."""
    import argparse as _a
    sub = _a.Namespace(**vars(args))
    sub.jmax = args.serve_jmax
    prob = make_problem(sub)
    jobs = prob.pair_jobs()
    rng = np.random.default_rng(args.seed + 17)
    order = [jobs[i] for i in rng.permutation(len(jobs))]
    gaps = rng.exponential(1.0 / args.serve_rate, size=len(order))
    with pkg.Engine(device) as eng:
        eng.load(prob, precision=precision, split_slices=args.slices)
        eng.serve_start(slots=args.serve_slots)
        eng.job_lines(eng.submit(*order[0]))  # first launch of every kernel
        eng.serve_reset_stats()
        ids = []
        t0 = time.perf_counter()
        due = t0
        for job, gap in zip(order, gaps):
            due += gap
            delay = due - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            ids.append(eng.submit(*job))
        for i in ids:
            eng.job_lines(i)
        makespan = time.perf_counter() - t0
        st = eng.serve_stats()
        eng.serve_stop()
    return {"workload": f"{args.workload} J<={args.serve_jmax} pair jobs", "jobs": len(order),
            "arrival": f"Poisson {args.serve_rate:g} jobs/s, random order",
            "slots": st["slots"], "precision": "split" if precision else "fp64",
            "latency_p50_s": st["latency_p50"], "latency_p99_s": st["latency_p99"],
            "latency_max_s": st["latency_max"], "latency_mean_s": st["latency_mean"],
            "queue_p50_s": st["queue_p50"], "queue_p99_s": st["queue_p99"],
            "makespan_s": makespan, "value": st["lines_filtered"] / makespan, "unit": METRIC,
            "lines_filtered": st["lines_filtered"], "lines_above_threshold": st["lines"],
            "failed": st["failed"], "evictions": st["evictions"],
            "budget_bytes": st["budget_bytes"], "peak_resident_bytes": st["peak_resident_bytes"]}


# ---------------------------------------------------------------- our arm
def main_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    pkg = G.load_package()
    prob = make_problem(args, rank)
    prec = pkg.GI_PREC_SPLIT if args.precision == "split" else pkg.GI_PREC_FP64

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    eng = pkg.Engine(local)
    eng.load(prob, precision=prec, split_slices=args.slices)
    # the warm-up steps also tune the split GEMM launch configurations
    import tempfile
    tune_path = args.tune_table or os.path.join(tempfile.gettempdir(),
                                                f"gi_tune_{os.getpid()}.txt")
    eng.set_tuning(1, tune_path)
    # the engine's launches go to this stream, so its CUDA events bracket them
    stream = torch.cuda.Stream(device=local)
    eng.set_stream(stream.cuda_stream)

    def timed_steps(k, fn):
        """Device seconds per step of k calls of fn, CUDA events on the stream."""
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        barrier()
        a.record(stream)
        out = None
        for _ in range(k):
            out = fn()
        b.record(stream)
        torch.cuda.synchronize()
        barrier()
        return a.elapsed_time(b) * 1e-3 / k, out

    for _ in range(args.warmup):
        eng.run(lines_on_device=True, graph=True)
    autotune = []
    if os.path.exists(tune_path):
        names = {"0": "one-pass", "1": "two-pass (split at s/2)", "2": "two-pass (split at s - s/2)",
                 "6": "grouped layout, two-pass (s/2)",
                 "7": "grouped layout, two-pass (s - s/2)", "8": "grouped layout, one-pass"}
        for line in open(tune_path).read().splitlines():
            s_, nA, nb, K, layout, kind, ga, ms = line.split()
            autotune.append({"digits": int(s_), "row_tiles": int(nA), "cols_bucket": 2 ** int(nb),
                             "K": int(K), "kernel": names[kind], "l2_group_mb": int(ga),
                             "ms": float(ms)})
    stats = []

    def one():
        eng.run(lines_on_device=True, graph=True)
        stats.append(eng.stats())

    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        dt, _ = timed_steps(args.steps, one)
        t1 = time.perf_counter()
    wall = (t1 - t0) / args.steps
    lines_pre = stats[-1]["nlines_filtered"]
    lines_post = stats[-1]["nlines"]
    launches = int(sum(s["kernel_launches"] for s in stats))

    # roofline of the dominant kernel: one more step with per-kernel events
    eng.run(lines_on_device=True, phase_timing=True)
    ps = eng.stats()
    sp = ps["seconds_phase"]
    lp = ps["launches_phase"]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    if args.precision == "split":
        # the dominant launch: the half-line-strength split GEMM (k_split_gemm_g),
        # one launch per step; digit-pair products x 2 x 3 x N x N x Y columns
        dom = "halfls_gemm"
        pairs = ps["flops_tensor"] / max(ps["flops_halfls"] + ps["flops_final"], 1.0)
        flops = pairs * ps["flops_halfls"]
        ncol = ps["flops_halfls"] / (6.0 * prob.N * prob.N)
        peak = peaks.get("bf16_tflops", 1900.0)
        achieved = flops / sp[dom] / 1e12 if sp[dom] else 0.0
        roof = {"bound": "tensor", "kernel": "k_split_gemm_g (tcgen05 bf16 digit GEMM, "
                                             "grouped digit layout, half line strength)",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak,
                "traffic": SPLIT_HALFLS_DRAM_BYTES_PER_COL * ncol / lp[dom],
                "traffic_source": "ncu dram__bytes_read+write of this kernel on the J<=4 part "
                                  "of the workload, scaled by Y columns",
                "algorithmic_tflop_per_launch": flops / lp[dom] / 1e12,
                "digit_pair_products": pairs,
                "both_gemms_tflops": ps["flops_tensor"] /
                (sp["halfls_gemm"] + sp["final_gemm"]) / 1e12,
                "peak_source": "MEASURED_PEAKS.json bf16_tflops (of measured)"
                if "bf16_tflops" in peaks else "fallback 1.9 PFLOP/s"}
    else:
        dom = "halfls_gemm"
        fp64_peak = pkg.measure_fp64_peak(local)  # TFLOP/s, DMMA m8n8k4, measured live
        achieved = ps["flops_halfls"] / sp[dom] / 1e12 if sp[dom] else 0.0
        roof = {"bound": "tensor", "kernel": "k_gemm_fp64_nt (FP64 DMMA, half line strength)",
                "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": achieved / fp64_peak, "traffic": None,
                "peak_source": "FP64 DMMA peak measured live by gi_measure_fp64_peak "
                               "(of measured); MEASURED_PEAKS.json has no FP64 entry"}
    roof["phase_seconds"] = {k: round(v, 6) for k, v in sp.items()}
    roof["phase_launches"] = lp
    roof["launch_avg_ms"] = 1e3 * sp[dom] / max(lp[dom], 1)

    # end to end through the C ABI from pinned host buffers
    e2e = None
    if not args.no_e2e:
        pin = {}
        mu = torch.from_numpy(prob.mu).pin_memory()
        for k, b in prob.blocks.items():
            pin[k] = torch.from_numpy(np.ascontiguousarray(b.vecs)).pin_memory()
        h2d = mu.numel() * 8 + sum(v.numel() * 8 for v in pin.values())
        ne = args.e2e_steps or args.steps

        parts = {"upload_ms": 0.0, "run_ms": 0.0}

        def step():
            t0 = time.perf_counter()
            eng.set_dipole(prob.N, mu.numpy())
            for (J, g), b in sorted(prob.blocks.items()):
                eng.set_block(J, g, pin[(J, g)].numpy(), b.energies, b.quanta)
            t1 = time.perf_counter()
            n = eng.run(lines_on_device=False, graph=True)
            parts["upload_ms"] += 1e3 * (t1 - t0)
            parts["run_ms"] += 1e3 * (time.perf_counter() - t1)
            return n

        step()
        parts["upload_ms"] = parts["run_ms"] = 0.0
        te, n = timed_steps(ne, step)
        st = eng.stats()
        e2e = {"value": world * st["nlines_filtered"] / te, "unit": METRIC,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(n * 80 + 16),
               "ms_per_step": 1e3 * te, "steps": ne,
               "host_wall_ms_per_step": {k: v / ne for k, v in parts.items()},
               "last_run_ms": {"wall": 1e3 * st["seconds_total"], "device": 1e3 * st["seconds_gpu"]}}

    # the same job with the dipole kept in host memory and streamed through
    # the device in four panels per half-ls GEMM (copies overlap the GEMMs)
    streamed = None
    if not args.no_stream:
        rows = -(-prob.N // 4)
        rows = -(-rows // 128) * 128
        eng.set_dipole_streamed(prob.N, prob.mu, panel_rows=rows)
        eng.run(lines_on_device=True)  # warm-up (and tuning of the panel GEMM shapes)
        ts, _ = timed_steps(1, lambda: eng.run(lines_on_device=True))
        ss = eng.stats()
        nr = ss["launches_phase"]["halfls_gemm"] // -(-prob.N // rows)  # GEMM rounds per step
        streamed = {"value": world * ss["nlines_filtered"] / ts, "unit": METRIC,
                    "ms_per_step": 1e3 * ts, "steps": 1, "warmup": 1, "panel_rows": rows,
                    "panels": -(-prob.N // rows), "rounds": int(nr),
                    "h2d_bytes_per_step": int(nr * 3 * prob.N * prob.N * 8),
                    "vs_resident": (ss["nlines_filtered"] / ts) / (lines_pre / dt),
                    "graph": "eager launches (a streamed dipole is not captured)"}
        eng.set_dipole(prob.N, prob.mu)

    # the plain FP64 GPU path on the same job, and per-line accuracy of the
    # split path against it on the J <= 3 part of the workload
    fp64 = accuracy = None
    if args.precision == "split" and not args.no_fp64:
        eng.set_params(prob.params, precision=pkg.GI_PREC_FP64)
        eng.run(lines_on_device=True, graph=True)
        tf, _ = timed_steps(1, lambda: eng.run(lines_on_device=True, graph=True))
        fs = eng.stats()
        fp64 = {"value": world * fs["nlines_filtered"] / tf, "unit": METRIC,
                "ms_per_step": 1e3 * tf, "steps": 1, "warmup": 1,
                "speedup_split_over_fp64": (lines_pre / dt) / (fs["nlines_filtered"] / tf)}
        eng.set_params(prob.params, precision=prec, split_slices=args.slices)
        accuracy = split_accuracy(pkg, prob, args.slices, local)

    serving = None
    if not args.no_serve and world == 1:
        serving = {"split": serve_bench(pkg, args, local, pkg.GI_PREC_SPLIT)}
        if not args.no_fp64:
            serving["fp64"] = serve_bench(pkg, args, local, pkg.GI_PREC_FP64)

    dt, lines_all, lines_all_post = across_ranks(dt, lines_pre, lines_post, "cuda")
    out = None
    if rank == 0:
        out = {"metric": METRIC, "value": lines_all / dt, "unit": METRIC,
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": 1e3 * dt, "wall_ms_per_step": 1e3 * wall,
               "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic",
               "config": config_of(args, prob),
               "lines_per_step": lines_pre, "lines_above_threshold_per_step": lines_post,
               "value_above_threshold": lines_all_post / dt,
               "gpu_launches": launches, "graph": "each step is one CUDA graph launch (captured "
               "in warm-up, replayed)", "autotune": autotune, "roofline": roof, "e2e": e2e,
               "fp64_path": fp64, "accuracy": accuracy, "serving": serving,
               "dipole_streamed": streamed,
               "clocks": clk.summary()}
        if world == 1 and not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(prob)
        print(json.dumps(out))
    eng.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return main_reference(args)
    return main_ours(args)


if __name__ == "__main__":
    sys.exit(main())

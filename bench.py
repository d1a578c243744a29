#!/usr/bin/env python
"""Throughput benchmark of the GB300 line-intensity engine.

Headline workload ``c3v_batched`` (the batched form): tetratomic C3v (A1, A2,
E), J = 0..40, Nvib = 3000, up to 1500 eigenvectors per (J, Gamma) under
12000 cm^-1 (blocks of ~1000 to 81000 functions, ~40 GB of vectors), every
dJ = 0, +-1 block pair, T = 500 K; seeded synthetic inputs of those shapes (no
TROVE checkpoints exist here).  All blocks stay resident in HBM.

A step is one batch of that job: the initial levels at positions
l % 10 == shard of the energy-sorted level table against every final level,
the split of initial levels the reference makes across devices
(cuda_host.cu:1174).  Steps cycle through the ten shards, so ten steps are one
whole job.  Metric: linestrengths/s, lines passing every filter before the
intensity threshold (1e-30 cm/molecule; the post-threshold rate beside it).

  value   inputs resident in HBM, lines kept on the device, CUDA-event time of
          K steps on the engine's stream, bracketed by synchronize (and a
          barrier across ranks); each step is one CUDA-graph launch
  e2e     the whole job through the C ABI from pinned host buffers: each e2e
          step uploads the dipole and every eigenvector block once, runs all
          shards and reads every line back to host memory (40-byte compact
          records); the digit planes of the new blocks are re-cut inside it
  roofline    the half-ls split GEMM (the dominant kernel): tensor-pipe rate of
          its bf16 digit products against the measured bf16 peak, its FP64-
          equivalent rate, and its DRAM traffic
  fp64_path   the plain FP64 GPU path and the split path on the same batch (one
          fortieth of the job)
  accuracy    per-line error of both paths against the CPU oracle (double-double
          checker) on a (J, J+1) sample of the workload
  legs    the other workloads: c2v_plain (config 2: split and FP64 jobs),
          c2v_precision (config 3: split and FP64 on one batch), serving (pair
          jobs through gi_serve_*), the dipole streamed from host memory
  cpu_baseline / --impl reference   the reference's algorithm restated in C
          (plain FP64, the oracle port; the reference has no CPU path) on all
          host cores, on the same bounded sample of the workload in both arms

Multi-GPU (torchrun): every rank runs an independent replica of the job with its
own seed (no collective on the data path), value = all ranks' lines / max time
("weak" scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as G  # noqa: E402

METRIC = "linestrengths/s"
THRESH_I = 1e-30  # cm/molecule
SHARDS = {"c3v_batched": 10}
# the CPU sample (both arms): one reference run (J, J+1) restricted to the
# lowest initial levels
CPU_SAMPLE = {"c3v_batched": ((20, 21), 2), "c2v_plain": ((9, 10), 8),
              "c2v_small": ((0, 1), 4), "c3v_small": ((1, 2), 4)}
# DRAM traffic of the half-line-strength split GEMM from one ncu capture of its
# first K segment (K = 2048) on a small case of the same Nvib (profiles/):
# bytes read per Y column per K element (the digit planes streamed past the
# tiles) and bytes written per Y column (Z).  A job's K runs in segments of
# 2048; each later segment re-reads Z to add to it.
SPLIT_HALFLS_TRAFFIC = {3000: {"read_per_col_k": 44108294656 / (47904 * 2048),
                               "write_per_col": 4468934656 / 47904,
                               "capture": "c3v_batched J <= 8, 47904 Y columns, K = 2048"}}


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c3v_batched")
    ap.add_argument("--jmax", type=int, default=None, help="restrict J to 0..jmax")
    ap.add_argument("--shards", type=int, default=None,
                    help="batches per job (a step is one batch); default 10 for c3v_batched")
    ap.add_argument("--precision", default="split", choices=["fp64", "split"])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--slices", type=int, default=0, help="bf16 digits per operand (split)")
    ap.add_argument("--e2e-steps", type=int, default=2, help="e2e steps (whole jobs)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64-path comparison")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-legs", action="store_true",
                    help="skip the other workloads (c2v_plain, c2v_precision, serving, streamed)")
    ap.add_argument("--legs", default="plain,precision,serving,streamed,halfls")
    ap.add_argument("--only", default=None,
                    help="run only these legs (comma list) and print their JSON, no headline")
    ap.add_argument("--serve-jobs", type=int, default=2000, help="serving: jobs (split path)")
    ap.add_argument("--serve-fp64-jobs", type=int, default=50,
                    help="serving: the first jobs of the stream again on the FP64 path")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="serving: Poisson jobs/s")
    ap.add_argument("--serve-slots", type=int, default=3)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--tune-table", default=None,
                    help="autotuner table file: read if present, extended and written")
    return ap.parse_args(argv)


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


def make_problem(args, rank=0, workload=None, jlist=None):
    G.load_package()
    from gpu_intensities_gb300 import synth
    kw = {}
    if jlist is not None:
        kw["jlist"] = list(jlist)
    elif args.jmax is not None:
        kw["jlist"] = list(range(args.jmax + 1))
    prob = synth.workload(workload or args.workload, seed=args.seed + rank, **kw)
    prob.params.thresh_intensity = THRESH_I
    return prob


def synth_block(b, vecs):
    """The same block with its vectors in another array."""
    from gpu_intensities_gb300 import synth
    return synth.Block(b.J, b.gamma, vecs, b.energies, b.quanta)


def nshards_of(args):
    return args.shards if args.shards else SHARDS.get(args.workload, 1)


def config_of(args, prob):
    vec_bytes = sum(b.vecs.nbytes for b in prob.blocks.values())
    return {"workload": args.workload, "sym": "C2v" if prob.sym_type == 1 else "C3v",
            "J": [min(prob.jlist), max(prob.jlist)], "Nvib": prob.N,
            "nvec_max_per_block": max(b.nvec for b in prob.blocks.values()),
            "nsize_max": max(b.nsize for b in prob.blocks.values()),
            "levels": int(sum(b.nvec for b in prob.blocks.values())),
            "eigenvector_bytes": int(vec_bytes), "T_K": prob.params.temperature,
            "shards_per_job": nshards_of(args),
            "step": "one shard: initial levels l % shards == step % shards of the level table, "
                    "every final level",
            "precision": args.precision, "thresh_intensity_cm_per_molecule": THRESH_I,
            "l2": f"inputs ({vec_bytes / 1e9:.1f} GB of eigenvectors) larger than L2",
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


# ---------------------------------------------------------------- samples
def sample_problem(args, workload):
    """The bounded sample of a workload: the two J of one reference run, with
    the initial levels restricted to the lowest few (lower energy window)."""
    (j0, j1), nlow = CPU_SAMPLE[workload]
    prob = make_problem(args, workload=workload, jlist=[j0, j1])
    e = np.sort(np.concatenate([b.energies for b in prob.blocks.values()]))
    cut = float(e[min(nlow, len(e)) - 1])
    prob.params.erange_lower = (prob.params.erange_lower[0], cut)
    return prob, (j0, j1), nlow


def run_cpu(prob, pair, threads, precise):
    O = G.load_oracle()
    t = time.perf_counter()
    lines = O.run_pair(prob, pair, None, nthreads=threads, precise=precise)
    return lines, time.perf_counter() - t


def cpu_baseline(args):
    prob, pair, nlow = sample_problem(args, args.workload)
    threads = os.cpu_count() or 1
    lines, dt = run_cpu(prob, pair, threads, precise=False)
    return {"value": len(lines) / dt, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{args.workload}: the reference run over J={pair[0]},{pair[1]} with the "
                      f"{nlow} lowest initial levels ({len(lines)} lines in {dt:.1f} s), the "
                      f"reference's algorithm restated in C, plain FP64, OpenMP"}


# ---------------------------------------------------------------- accuracy
def _sorted_keyed(lines):
    keys = ("jI", "gammaI", "recI", "jF", "gammaF", "recF")
    return lines[np.lexsort(tuple(lines[k] for k in reversed(keys)))], keys


def compare_lines(got, ref):
    """Identical selection and the per-line relative error of S against the
    oracle, on every line (all lines here are above the intensity threshold)."""
    g, keys = _sorted_keyed(got)
    r, _ = _sorted_keyed(ref)
    same = len(g) == len(r) and all(np.array_equal(g[k], r[k]) for k in keys)
    out = {"lines": int(len(r)), "identical_selection": bool(same)}
    if same and len(r):
        rel = np.abs(g["S"] - r["S"]) / np.abs(r["S"])
        out.update({"rel_err_S_max": float(rel.max()), "rel_err_S_p99": float(np.quantile(rel, 0.99)),
                    "rel_err_I_max": float((np.abs(g["I"] - r["I"]) / np.abs(r["I"])).max())})
    return out


def accuracy_vs_oracle(pkg, args, device, workload):
    """Both GPU paths against the CPU oracle (double-double checker) on the
    bounded sample of the workload."""
    prob, pair, nlow = sample_problem(args, workload)
    ref, dt = run_cpu(prob, pair, os.cpu_count() or 1, precise=True)
    out = {"sample": f"{workload}: reference run J={pair[0]},{pair[1]}, the {nlow} lowest initial "
                     f"levels, every line above the intensity threshold",
           "oracle_seconds": dt}
    for name, prec in (("split", pkg.GI_PREC_SPLIT), ("fp64", pkg.GI_PREC_FP64)):
        for refine in (0, 1 << 20):
            with pkg.Engine(device) as e:
                e.load(prob, precision=prec, split_slices=args.slices)
                e.set_refine(refine)
                e.run()
                got = pkg.keyed(e.lines(), e.levels())
                st = e.stats()
            r = compare_lines(got, ref)
            r.update({"doubtful_lines": st["nlines_doubtful"], "refined_lines": st["nlines_refined"]})
            out[name + ("_refined" if refine else "")] = r
    return out


# ---------------------------------------------------------------- reference arm
def main_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    prob, pair, nlow = sample_problem(args, args.workload)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        run_cpu(prob, pair, threads, precise=False)
    tot_n, tot_t = 0, 0.0
    for _ in range(args.steps):
        lines, dt = run_cpu(prob, pair, threads, precise=False)
        tot_n += len(lines)
        tot_t += dt
    v = tot_n / tot_t
    cfg = {"workload": args.workload, "sample_of": args.workload, "J": list(pair),
           "initial_levels": nlow, "precision": "fp64",
           "thresh_intensity_cm_per_molecule": THRESH_I, "seed": args.seed}
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC,
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": cfg,
           "cpu_baseline": {"value": v, "unit": METRIC, "cores": threads, "kind": "port",
                            "sample": f"the reference's algorithm restated in C (plain FP64, "
                                      f"OpenMP; the reference has no CPU path) over "
                                      f"J={pair[0]},{pair[1]} with the {nlow} lowest initial "
                                      f"levels per step"},
           "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


# ---------------------------------------------------------------- serving
def serve_stream(pkg, pool, jobs, gaps, device, precision, args):
    """Submits the jobs with their Poisson gaps to a serving context over the
    pool; a reaper thread waits for every job (latency = submit -> lines in
    host memory) and releases it.  Returns the server's statistics."""
    with pkg.Engine(device) as eng:
        eng.load(pool, precision=precision, split_slices=args.slices)
        eng.serve_start(slots=args.serve_slots, budget=int(args.serve_budget_gb * 1e9))
        w = eng.submit(*jobs[0])  # first launch of every kernel
        eng.wait(w)
        eng.release(w)
        eng.serve_reset_stats()
        ids, errors = [], []
        lock = threading.Lock()
        done = threading.Event()

        def reap():
            k = 0
            while True:
                with lock:
                    nxt = ids[k] if k < len(ids) else None
                if nxt is None:
                    if done.is_set():
                        with lock:
                            if k >= len(ids):
                                return
                    time.sleep(0.001)
                    continue
                info = eng.wait(nxt, check=False)
                if info["state"] != pkg.GI_JOB_DONE:
                    errors.append(info["status"])
                eng.release(nxt)
                k += 1

        th = threading.Thread(target=reap, daemon=True)
        t0 = time.perf_counter()
        th.start()
        due = t0
        for job, gap in zip(jobs, gaps):
            due += gap
            delay = due - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            i = eng.submit(*job)
            with lock:
                ids.append(i)
        done.set()
        th.join()
        makespan = time.perf_counter() - t0
        st = eng.serve_stats()
        eng.serve_stop()
    st["makespan_s"] = makespan
    st["reaped_failures"] = len(errors)
    return st


def serving_leg(pkg, args, device, base):
    """Config 5: pair jobs drawn from the batched C3v generator (initial block
    dimensions log-uniform in 500..80k, 100..2000 vectors per block), Poisson
    arrivals, blocks resident under an HBM budget with LRU eviction of blocks
    (to pinned host memory) and of cached half line strengths."""
    from gpu_intensities_gb300 import synth
    if base is None:
        base = make_problem(args, workload="c3v_batched")
    pool = synth.serving_pool(base, seed=args.seed + 40)
    jobs, gaps = synth.serving_jobs(pool, seed=args.seed + 41, njobs=args.serve_jobs,
                                    rate=args.serve_rate)
    out = {"workload": "serving: pool of every C3v J=0..40 block (Nvib=3000) with 100..2000 "
                       "vectors (log-uniform), pair jobs with initial block dimension "
                       "log-uniform in 500..80k",
           "pool_vector_bytes": int(sum(b.vecs.nbytes for b in pool.blocks.values())),
           "arrival": f"Poisson {args.serve_rate:g} jobs/s", "slots": args.serve_slots,
           "budget_bytes": int(args.serve_budget_gb * 1e9)}
    for name, prec, n in (("split", pkg.GI_PREC_SPLIT, args.serve_jobs),
                          ("fp64", pkg.GI_PREC_FP64, args.serve_fp64_jobs)):
        if n <= 0:
            continue
        st = serve_stream(pkg, pool, jobs[:n], gaps[:n], device, prec, args)
        out[name] = {"jobs": n, "completed": st["completed"], "failed": st["failed"],
                     "latency_p50_s": st["latency_p50"], "latency_p99_s": st["latency_p99"],
                     "latency_max_s": st["latency_max"], "latency_mean_s": st["latency_mean"],
                     "queue_p50_s": st["queue_p50"], "queue_p99_s": st["queue_p99"],
                     "makespan_s": st["makespan_s"],
                     "value": st["lines_filtered"] / st["makespan_s"], "unit": METRIC,
                     "lines_filtered": st["lines_filtered"], "lines_above_threshold": st["lines"],
                     "block_evictions": st["evictions"], "block_restores": st["restores"],
                     "zcache_hits": st["zcache_hits"], "zcache_misses": st["zcache_misses"],
                     "zcache_evictions": st["zcache_evictions"],
                     "peak_resident_bytes": st["peak_resident_bytes"]}
    if "fp64" in out:
        out["fp64"]["note"] = (f"the first {args.serve_fp64_jobs} jobs of the same stream: the "
                               "FP64 path cannot keep up with 200 jobs/s, so its queue grows")
    return out


# ---------------------------------------------------------------- helpers
class Timer:
    """Device seconds of a callable's launches: CUDA events on the engine's
    stream, bracketed by synchronize and a barrier across ranks."""

    def __init__(self, torch, stream, barrier):
        self.torch, self.stream, self.barrier = torch, stream, barrier

    def __call__(self, k, fn):
        torch = self.torch
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        self.barrier()
        a.record(self.stream)
        out = [fn(i) for i in range(k)]
        b.record(self.stream)
        torch.cuda.synchronize()
        self.barrier()
        return a.elapsed_time(b) * 1e-3, out


def split_roofline(prob, ps, peaks):
    """The dominant kernel of the split path: the half-line-strength digit GEMM
    (k_split_gemm_g, one launch per round)."""
    sp, lp = ps["seconds_phase"], ps["launches_phase"]
    dom = "halfls_gemm"
    pairs = ps["flops_tensor"] / max(ps["flops_halfls"] + ps["flops_final"], 1.0)
    flops = pairs * ps["flops_halfls"]
    ncol = ps["flops_halfls"] / (6.0 * prob.N * prob.N)
    peak = peaks.get("bf16_tflops", 1900.0)
    achieved = flops / sp[dom] / 1e12 if sp[dom] else 0.0
    tr = SPLIT_HALFLS_TRAFFIC.get(prob.N)
    traffic = None
    if tr:
        kp = -(-prob.N // 64) * 64
        nseg = -(-kp // 2048)
        step_bytes = ncol * (tr["read_per_col_k"] * kp + tr["write_per_col"] * (2 * nseg - 1))
        traffic = step_bytes / max(lp[dom], 1)
    algo = ncol * (9 * 2 * (-(-prob.N // 64) * 64) + 3 * prob.N * 8) / max(lp[dom], 1)
    return {"bound": "tensor", "kernel": "k_split_gemm_g (tcgen05 bf16 digit GEMM, grouped digit "
                                         "layout, half line strength)",
            "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": traffic,
            "traffic_source": (f"ncu dram__bytes_read+write of this kernel on {tr['capture']}, "
                               "scaled to the launch by Y columns and K (reads) and by Y columns "
                               "(writes, and the re-read of Z by later K segments)")
            if tr else "not captured for this Nvib",
            "algorithmic_bytes_per_launch": algo,
            "algorithmic_bytes_meaning": "Y digit planes (9 x 2 B x Kp per column) read once and "
                                         "Z (3 x N doubles per column) written once, per launch "
                                         "averaged over the step's launches; the dipole's digit "
                                         "planes (0.5 GB) are re-read per L2 raster group",
            "achieved_meaning": "bf16 tensor-pipe rate: digit-pair products x 2 x M x N x K",
            "tensor_tflop_per_launch": flops / max(lp[dom], 1) / 1e12,
            "digit_pair_products": pairs,
            "fp64_equivalent_tflops": ps["flops_halfls"] / sp[dom] / 1e12 if sp[dom] else 0.0,
            "fp64_algorithmic_tflop_per_launch": ps["flops_halfls"] / max(lp[dom], 1) / 1e12,
            "both_gemms_tflops": ps["flops_tensor"] / (sp["halfls_gemm"] + sp["final_gemm"]) / 1e12,
            "peak_source": "MEASURED_PEAKS.json bf16_tflops (of measured)"
            if "bf16_tflops" in peaks else "fallback 1.9 PFLOP/s",
            "phase_seconds": {k: round(v, 6) for k, v in sp.items()},
            "phase_launches": lp, "launch_avg_ms": 1e3 * sp[dom] / max(lp[dom], 1),
            "launch_unit": "one round's half-ls GEMM: its K segments (2048, then the rest) as "
                           "consecutive kernel launches; achieved, traffic and launch_avg_ms "
                           "are per such launch"}


# ---------------------------------------------------------------- legs
def leg_c2v_plain(pkg, args, device, timer_of):
    """Config 2: the whole C2v J = 0..10 job per step, split and FP64."""
    import torch
    prob = make_problem(args, workload="c2v_plain")
    out = {"workload": "c2v_plain: C2v, J=0..10, Nvib=2000, <=1000 vectors per (J, Gamma); one "
                       "step = the whole job"}
    with pkg.Engine(device) as eng:
        stream = torch.cuda.Stream(device=device)
        eng.set_stream(stream.cuda_stream)
        timer = timer_of(stream)
        eng.load(prob, precision=pkg.GI_PREC_SPLIT, split_slices=args.slices)
        for _ in range(3):
            eng.run(lines_on_device=True, graph=True)
        dt, n = timer(3, lambda i: (eng.run(lines_on_device=True, graph=True),
                                    eng.stats()["nlines_filtered"])[1])
        out["split"] = {"value": sum(n) / dt, "unit": METRIC, "ms_per_step": 1e3 * dt / 3,
                        "steps": 3, "lines_per_step": n[-1]}
        eng.set_params(prob.params, precision=pkg.GI_PREC_FP64)
        eng.run(lines_on_device=True, graph=True)
        dt, n = timer(1, lambda i: (eng.run(lines_on_device=True, graph=True),
                                    eng.stats()["nlines_filtered"])[1])
        out["fp64"] = {"value": sum(n) / dt, "unit": METRIC, "ms_per_step": 1e3 * dt, "steps": 1}
    out["speedup_split_over_fp64"] = out["split"]["value"] / out["fp64"]["value"]
    return out


def leg_c2v_precision(pkg, args, device, timer_of):
    """Config 3: C2v J = 20 -> 21, Nvib = 5000, 2000 vectors per block of ~26k,
    log-uniform dipole; split and FP64 on the same batch (one tenth of the
    initial levels)."""
    import torch
    prob = make_problem(args, workload="c2v_precision")
    S = 10
    out = {"workload": "c2v_precision: C2v, J=20,21, Nvib=5000, 2000 vectors per block, nsize "
                       f"~26k, dipole log-uniform 1e-8..1; one step = shard 0 of {S}"}
    with pkg.Engine(device) as eng:
        stream = torch.cuda.Stream(device=device)
        eng.set_stream(stream.cuda_stream)
        timer = timer_of(stream)
        for name, prec, k in (("split", pkg.GI_PREC_SPLIT, 3), ("fp64", pkg.GI_PREC_FP64, 1)):
            if name == "split":
                eng.load(prob, precision=prec, split_slices=args.slices)
            else:
                eng.set_params(prob.params, precision=prec)
            eng.run(lines_on_device=True, graph=True, shard=0, nshards=S)
            dt, n = timer(k, lambda i: (eng.run(lines_on_device=True, graph=True, shard=0,
                                                nshards=S), eng.stats()["nlines_filtered"])[1])
            out[name] = {"value": sum(n) / dt, "unit": METRIC, "ms_per_step": 1e3 * dt / k,
                         "steps": k, "lines_per_step": n[-1]}
    out["speedup_split_over_fp64"] = out["split"]["value"] / out["fp64"]["value"]
    return out


def leg_half_ls(pkg, args, device, timer_of, peaks):
    """The kernel-level drop-in for do_1st_half_ls (gi_half_ls): the half line
    strength of one initial vector of C2v J = 10 (Nvib = 2000, 22 (k, tau)
    slots) towards J = 10, per call.  The split path is one pass over the
    dipole's digit planes (the narrow digit GEMM, K split over the SMs); the
    FP64 path is the DMMA GEMM."""
    import torch
    prob = make_problem(args, workload="c2v_plain", jlist=[9, 10])
    blk = prob.blocks[(10, 0)]
    DF = prob.bases[10].Maxcontracts
    N = prob.N
    Kp = -(-N // 64) * 64
    Mpad = -(-N // 128) * 128
    digit_bytes = 3 * Mpad * Kp * 9 * 2
    out = {"workload": f"gi_half_ls: one C2v J=10 vector (nsize {blk.nsize}) towards J=10, Nvib={N}",
           "dipole_fp64_bytes": 3 * N * N * 8, "dipole_digit_bytes": digit_bytes}
    for name, prec in (("split", pkg.GI_PREC_SPLIT), ("fp64", pkg.GI_PREC_FP64)):
        with pkg.Engine(device) as eng:
            stream = torch.cuda.Stream(device=device)
            eng.set_stream(stream.cuda_stream)
            timer = timer_of(stream)
            eng.load(prob, precision=prec)
            for w in range(3):
                eng.half_ls(10, 0, 0, 10, blk.vecs[w], DF)
            k = 20
            dt, _ = timer(k, lambda i: eng.half_ls(10, 0, 0, 10, blk.vecs[i % blk.nvec], DF))
            per = dt / k
            r = {"us_per_call": 1e6 * per, "calls": k,
                 "note": "device time per call on the engine's stream (Y build, GEMM, stencil, "
                         "copies of the vector and the result)"}
            if name == "split":
                r["digit_gb_per_s_whole_call"] = digit_bytes / per / 1e9
            out[name] = r
    out["speedup_split_over_fp64"] = out["fp64"]["us_per_call"] / out["split"]["us_per_call"]
    return out


def leg_streamed(pkg, eng, prob, timer, S, value_rate):
    """The headline batch with the dipole kept in host memory and streamed
    through the device in four panels per half-ls GEMM (copies overlap)."""
    rows = -(-prob.N // 4)
    rows = -(-rows // 128) * 128
    eng.set_dipole_streamed(prob.N, prob.mu, panel_rows=rows)
    eng.run(lines_on_device=True, shard=0, nshards=S)
    ts, n = timer(1, lambda i: (eng.run(lines_on_device=True, shard=0, nshards=S),
                                eng.stats())[1])
    ss = n[-1]
    nr = ss["launches_phase"]["halfls_gemm"] // -(-prob.N // rows)
    eng.set_dipole(prob.N, prob.mu)
    return {"value": ss["nlines_filtered"] / ts, "unit": METRIC, "ms_per_step": 1e3 * ts,
            "steps": 1, "panel_rows": rows, "panels": -(-prob.N // rows), "rounds": int(nr),
            "h2d_bytes_per_step": int(nr * 3 * prob.N * prob.N * 8),
            "vs_resident": (ss["nlines_filtered"] / ts) / value_rate,
            "graph": "eager launches (a streamed dipole is not captured)"}


# ---------------------------------------------------------------- our arm
def main_only(args):
    """Selected legs alone (profiling runs): their JSON, no headline."""
    import torch
    pkg = G.load_package()
    local = dist_env()[2]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass

    def timer_of(stream):
        return Timer(torch, stream, lambda: None)

    out = {}
    for leg in args.only.split(","):
        if leg == "halfls":
            out[leg] = leg_half_ls(pkg, args, local, timer_of, peaks)
        elif leg == "plain":
            out[leg] = leg_c2v_plain(pkg, args, local, timer_of)
        elif leg == "precision":
            out[leg] = leg_c2v_precision(pkg, args, local, timer_of)
        elif leg == "serving":
            out[leg] = serving_leg(pkg, args, local, None)
        else:
            raise SystemExit(f"unknown leg {leg}")
    print(json.dumps(out))
    return 0


def main_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    pkg = G.load_package()
    prec = pkg.GI_PREC_SPLIT if args.precision == "split" else pkg.GI_PREC_FP64
    S = nshards_of(args)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def timer_of(stream):
        return Timer(torch, stream, barrier)

    t_setup = time.perf_counter()
    prob = make_problem(args, rank)
    cfg = config_of(args, prob)
    eng = pkg.Engine(local)
    eng.load(prob, precision=prec, split_slices=args.slices)
    setup_s = time.perf_counter() - t_setup
    # the warm-up steps also tune the split GEMM launch configurations
    tune_path = args.tune_table or os.path.join(tempfile.gettempdir(),
                                                f"gi_tune_{os.getpid()}.txt")
    eng.set_tuning(1, tune_path)
    # the engine's launches go to this stream, so its CUDA events bracket them
    stream = torch.cuda.Stream(device=local)
    eng.set_stream(stream.cuda_stream)
    timer = timer_of(stream)

    def step(i):
        eng.run(lines_on_device=True, graph=True, shard=i % S, nshards=S)
        return eng.stats()

    for w in range(args.warmup):
        step(w)
    eng.set_tuning(0, tune_path)  # tuned: later shards are captured on their first run
    autotune = []
    if os.path.exists(tune_path):
        names = {"0": "one-pass", "1": "two-pass (split at s/2)", "2": "two-pass (split at s - s/2)",
                 "6": "grouped layout, two-pass (s/2)", "7": "grouped layout, two-pass (s - s/2)",
                 "8": "grouped layout, one-pass",
                 "9": "grouped layout, two-pass, 2-SM pair (cta_group::2, 256-row tiles)"}
        for line in open(tune_path).read().splitlines():
            s_, nA, nb, K, layout, kind, ga, ms = line.split()
            autotune.append({"digits": int(s_), "row_tiles": int(nA), "cols_bucket": 2 ** int(nb),
                             "K": int(K), "kernel": names.get(kind, kind), "l2_group_mb": int(ga),
                             "ms": float(ms)})

    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        dt, stats = timer(args.steps, step)
        t1 = time.perf_counter()
    wall = (t1 - t0) / args.steps
    doubtful = int(sum(s["nlines_doubtful"] for s in stats))
    handed = int(sum(s["nlines_handed"] for s in stats))
    lines_pre = int(sum(s["nlines_filtered"] for s in stats))
    lines_post = int(sum(s["nlines"] for s in stats))
    launches = int(sum(s["kernel_launches"] for s in stats))
    value_rate = lines_pre / dt

    # roofline of the dominant kernel: one more step with per-kernel events
    eng.run(lines_on_device=True, phase_timing=True, shard=0, nshards=S)
    ps = eng.stats()
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    if args.precision == "split":
        roof = split_roofline(prob, ps, peaks)
    else:
        sp, lp = ps["seconds_phase"], ps["launches_phase"]
        fp64_peak = pkg.measure_fp64_peak(local)  # TFLOP/s, DMMA m8n8k4, measured live
        achieved = ps["flops_halfls"] / sp["halfls_gemm"] / 1e12 if sp["halfls_gemm"] else 0.0
        roof = {"bound": "tensor", "kernel": "k_gemm_fp64_nt (FP64 DMMA, half line strength)",
                "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": achieved / fp64_peak, "traffic": None,
                "peak_source": "FP64 DMMA peak measured live by gi_measure_fp64_peak "
                               "(of measured); MEASURED_PEAKS.json has no FP64 entry",
                "phase_seconds": sp, "phase_launches": lp}
    roof["measured_on"] = f"shard 0 of {S}, per-kernel CUDA events on the engine's stream"

    # end to end through the C ABI from pinned host buffers.  One e2e step is
    # the whole job as a caller runs it: upload the dipole and every block,
    # run every shard (each reads its lines back to host memory as compact
    # records while it computes), so the uploads are paid once per job
    e2e = None
    if not args.no_e2e:
        # the job's inputs in page-locked host memory (cudaHostAlloc through
        # torch), as a caller that owns pinned buffers hands them over
        # (each block's pageable array is dropped once its pinned copy exists,
        # so the host holds the job once)
        host = {"mu": torch.from_numpy(prob.mu).pin_memory().numpy()}
        for key, b in sorted(prob.blocks.items()):
            host[key] = torch.from_numpy(b.vecs).pin_memory().numpy()
            prob.blocks[key] = synth_block(b, host[key])
        h2d = sum(a.nbytes for a in host.values())
        parts = {"upload_ms": 0.0, "run_ms": 0.0, "dipole_ms": 0.0}
        d2h = []
        slowest = []

        def e2e_step(i):
            ta = time.perf_counter()
            eng.set_dipole(prob.N, host["mu"])
            parts["dipole_ms"] += 1e3 * (time.perf_counter() - ta)
            for (J, g), b in sorted(prob.blocks.items()):
                t = time.perf_counter()
                eng.set_block(J, g, host[(J, g)], b.energies, b.quanta)
                slowest.append((time.perf_counter() - t, b.vecs.nbytes, J, g))
            tb = time.perf_counter()
            n_pre, nbytes = 0, 0
            for sh in range(S):
                n = eng.run(lines_on_device=False, graph=True, shard=sh, nshards=S, compact=True)
                nbytes += n * 40 + 32  # compact records + the run's line counters
                n_pre += eng.stats()["nlines_filtered"]
            parts["upload_ms"] += 1e3 * (tb - ta)
            parts["run_ms"] += 1e3 * (time.perf_counter() - tb)
            d2h.append(nbytes)
            return n_pre

        e2e_step(0)
        for k in parts:
            parts[k] = 0.0
        d2h.clear()
        slowest.clear()
        ne = args.e2e_steps
        te, n = timer(ne, e2e_step)
        del host
        e2e = {"value": world * sum(n) / te, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(np.mean(d2h)), "ms_per_step": 1e3 * te / ne,
               "steps": ne, "step": f"one whole job: uploads, then all {S} shards",
               "value_over_device_value": (sum(n) / te) / value_rate,
               "host_memory": "page-locked (cudaHostAlloc)",
               "host_wall_ms_per_step": {k: v / ne for k, v in parts.items()},
               "upload_gb_per_s": h2d / (parts["upload_ms"] / ne * 1e-3),
               "slowest_block_uploads": [{"s": round(t, 4), "bytes": int(nb), "J": J, "gamma": g}
                                         for t, nb, J, g in sorted(slowest, reverse=True)[:4]],
               "note": "each step uploads the dipole and every block from page-locked host "
                       "memory, re-cuts the digit planes, and reads every line of every shard "
                       "back as 40-byte gi_line_compact records (GI_RUN_COMPACT_LINES)"}

    # the plain FP64 GPU path and the split path on the same batch
    fp64 = None
    if args.precision == "split" and not args.no_fp64:
        S4 = 4 * S
        res = {}
        for name, p in (("split", pkg.GI_PREC_SPLIT), ("fp64", pkg.GI_PREC_FP64)):
            eng.set_params(prob.params, precision=p, split_slices=args.slices)
            eng.run(lines_on_device=True, graph=True, shard=0, nshards=S4)
            tf, n = timer(1, lambda i: (eng.run(lines_on_device=True, graph=True, shard=0,
                                                nshards=S4), eng.stats()["nlines_filtered"])[1])
            res[name] = {"value": world * n[0] / tf, "unit": METRIC, "ms_per_step": 1e3 * tf,
                         "lines": n[0]}
        eng.set_params(prob.params, precision=prec, split_slices=args.slices)
        fp64 = {"batch": f"shard 0 of {S4} of the job (one fortieth of the initial levels, every "
                         f"final level)", "fp64": res["fp64"], "split": res["split"],
                "speedup_split_over_fp64": res["split"]["value"] / res["fp64"]["value"]}

    streamed = None
    if not args.no_legs and "streamed" in args.legs and world == 1:
        streamed = leg_streamed(pkg, eng, prob, timer, S, value_rate)
    eng.close()
    # the serving pool reuses the headline's dipole and bases (blocks regenerated)
    serve_base = None
    if args.workload == "c3v_batched" and args.jmax is None:
        from gpu_intensities_gb300 import synth as _synth
        serve_base = _synth.Problem(prob.sym_type, prob.N, prob.mu, prob.bases, {}, prob.params,
                                    name=prob.name)
    del prob

    legs = {}
    if not args.no_legs and world == 1:
        if "plain" in args.legs and args.workload != "c2v_plain":
            legs["c2v_plain"] = leg_c2v_plain(pkg, args, local, timer_of)
        if "precision" in args.legs and args.workload != "c2v_precision":
            legs["c2v_precision"] = leg_c2v_precision(pkg, args, local, timer_of)
        if "serving" in args.legs:
            legs["serving"] = serving_leg(pkg, args, local, serve_base)
        if "halfls" in args.legs:
            legs["half_ls_vector"] = leg_half_ls(pkg, args, local, timer_of, peaks)
    accuracy = None
    if not args.no_accuracy and world == 1 and args.workload in CPU_SAMPLE:
        accuracy = accuracy_vs_oracle(pkg, args, local, args.workload)

    dt, lines_all, lines_all_post = across_ranks(dt, lines_pre, lines_post, "cuda")
    if rank == 0:
        out = {"metric": METRIC, "value": lines_all / dt, "unit": METRIC,
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": 1e3 * dt / args.steps, "wall_ms_per_step": 1e3 * wall,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "split-bf16x9" if args.precision == "split" and args.slices in (0, 9)
               else (f"split-bf16x{args.slices}" if args.precision == "split" else "f64"),
               "dtype_note": "bf16 digit products with exact integer accumulation, FP64 "
                             "epilogue (S, A, I, filters in FP64)" if args.precision == "split"
               else "FP64 throughout",
               "data": "synthetic", "config": cfg,
               "lines_per_step": lines_pre / args.steps,
               "value_above_threshold": lines_all_post / dt,
               "gpu_launches": launches,
               "exact_reevaluation": {
                   "threshold_band_lines": handed, "doubtful_lines": doubtful,
                   "doubtful_fraction": doubtful / max(lines_post, 1),
                   "note": "lines within their error of a threshold are re-evaluated in "
                           "double-double before the keep decision; doubtful lines (moment "
                           "cancelled far below its column, estimated error past the target) "
                           "keep the GEMM path's accuracy here (gi_set_refine 0); the accuracy "
                           "block shows both settings against the oracle"},
               "graph": "each step is one CUDA graph launch (one graph per shard)",
               "setup_s": setup_s, "autotune": autotune, "roofline": roof, "e2e": e2e,
               "fp64_path": fp64, "accuracy": accuracy, "dipole_streamed": streamed,
               "legs": legs, "clocks": clk.summary()}
        if world == 1 and not args.no_cpu_baseline and args.workload in CPU_SAMPLE:
            out["cpu_baseline"] = cpu_baseline(args)
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return main_reference(args)
    if args.only:
        return main_only(args)
    return main_ours(args)


if __name__ == "__main__":
    sys.exit(main())

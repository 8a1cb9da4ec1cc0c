#!/usr/bin/env python3
"""Benchmark of the greedy clustering hot path on GB300.

Workload: the 1,000,000-sequence DNA configuration (20,000 ancestors, lengths
Normal(1450, 120) clipped to [900, 2000], substitutions U[0, 0.20], indels
1-3 at 5% of that rate), similarity 0.85, word length 5; generated in memory
by the seeded generator (no public dataset).  One step = S greedy iterations
(each: longest unclustered sequence becomes the representative, every
unclustered sequence is filtered and aligned against it, members join) run by
the device-side driver; the run continues from step to step.

value  = candidate sequences screened per second (sum over the timed
         iterations of the unclustered-set size), device time from CUDA events
         on the library's stream, max over ranks, summed over ranks.
e2e    = the same metric through the C ABI with host buffers: per step
         ngia_open (database host-to-device from pinned memory), S iterations,
         results device-to-host, close.
Multi-GPU: independent replicas (the path has no exchange step on one node).

`--impl reference` times the reference algorithm's CPU restatement (the
oracle; the reference's own CPU path is a SYCL build that cannot be compiled
here) on the host cores, one greedy iteration per step.
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "ngia-metax_gb300"))
sys.path.insert(0, str(ROOT))

METRIC = "seqs/sec (candidate sequences screened by the greedy clustering loop, bit-exact)"
UNIT = "candidate seqs/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--iters-per-step", type=int, default=32)
    ap.add_argument("--similarity", type=float, default=0.85)
    ap.add_argument("--word", type=int, default=5)
    ap.add_argument("--workload", default="dna_1m",
                    help="dna_small | dna_1m | protein_200k | batch256 | serve | dna_1m_whole")
    ap.add_argument("--batch-jobs", type=int, default=256)
    ap.add_argument("--batch-max-seqs", type=int, default=200000)
    ap.add_argument("--batch-autotune", type=int, default=0,
                    help="batch workloads: ngia_batch_autotune with this many iterations per setting first (0: off)")
    ap.add_argument("--batch-iters", type=int, default=-1,
                    help="batch256: greedy iterations per job and step (-1: --iters-per-step, 0: whole jobs)")
    ap.add_argument("--serve-batches", type=int, default=200)
    ap.add_argument("--serve-rate", type=float, default=200.0, help="Poisson arrivals, batches per second")
    ap.add_argument("--serve-slots", type=int, default=16)
    ap.add_argument("--n-seqs", type=int, default=0, help="override the sequence count (testing only)")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--mode", default="graph", choices=["graph", "plain"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-drivers", action="store_true", help="skip the whole-job graph vs plain comparison")
    ap.add_argument("--skip-secondary", action="store_true",
                    help="skip the sub-results of the other configurations (protein, serving, reference GPU)")
    ap.add_argument("--autotune", type=int, default=4, help="iterations per setting tried by ngia_autotune (0: off)")
    ap.add_argument("--sweep", default="0.8,0.9,0.95,0.99",
                    help="comma-separated similarities to time as well ('' = none)")
    ap.add_argument("--sweep-steps", type=int, default=2)
    ap.add_argument("--whole-mode", default="spec", choices=["spec", "graph", "plain"],
                    help="dna_1m_whole: the driver form that runs the whole job")
    ap.add_argument("--whole-chunk", type=int, default=8192, help="dna_1m_whole: representatives per step call")
    ap.add_argument("--whole-probe", type=int, default=64,
                    help="dna_1m_whole: iterations of each form timed from every checkpoint")
    ap.add_argument("--cpu-only", action="store_true",
                    help="replica plumbing with the CPU oracle as the engine (tests; no GPU)")
    return ap.parse_args()


# ---- distributed replicas ------------------------------------------------------
class Dist:
    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def reduce(self, value: float, op: str) -> float:
        if not self.pg:
            return value
        import torch

        t = torch.tensor([value], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX if op == "max" else self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---- clocks during the timed region -----------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                try:
                    rows.append((float(f[1]), float(f[2]), float(f[3]), f[5:9]))
                except ValueError:
                    pass
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k, v in enumerate(r[3]) if v.lower().startswith("active")})
        load = [r for r in rows if r[2] > 200.0] or rows
        return {"sm_mhz": statistics.median(r[0] for r in load), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": reasons}


def repo_libraries() -> list[str]:
    """Shared libraries of this repository mapped into the process."""
    try:
        maps = Path("/proc/self/maps").read_text().splitlines()
    except OSError:
        return []
    root = str(ROOT)
    return sorted({ln.split()[-1][len(root) + 1:] for ln in maps
                   if ln.split()[-1].startswith(root) and ".so" in ln.split()[-1]})


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs"), "source": "of measured"}
    return {"hbm_gbs": 6800.0, "source": "of fallback"}


def make_db(args):
    import ngia

    cfg = dict(ngia.CONFIGS[args.workload])
    if args.n_seqs:
        cfg["n_seqs"] = args.n_seqs
    seqs = ngia.synth(**cfg, seed=args.seed)
    db = ngia.DB.pack(cfg["type"], seqs, seqs.off)
    seqs.close()
    return db, cfg


def workload_desc(args, cfg, db_bytes: int | None = None) -> dict:
    dist = (f"~N({cfg['len_a']:.0f},{cfg['len_b']:.0f})" if cfg.get("len_dist", 0) == 0 else
            f"log-normal(median {cfg['len_a']:.0f}, sigma {cfg['len_b']:g})")
    out = {"workload": f"{args.workload}: {cfg['n_seqs']:,} {'DNA' if cfg['type'] == 0 else 'protein'} "
                       f"sequences, {cfg['n_ancestors']:,} ancestors, lengths {dist} clipped "
                       f"[{cfg['len_min']},{cfg['len_max']}], s={args.similarity}, w={args.word}",
           "iters_per_step": args.iters_per_step, "similarity": args.similarity, "word_length": args.word,
           "driver": args.mode, "seed": args.seed}
    if db_bytes is not None:
        big = db_bytes > 129e6
        out["l2"] = (f"inputs {'larger' if big else 'smaller'} than L2 (database {db_bytes / 1e6:.0f} MB vs "
                     f"129 MB L2)")
    return out


# ---- reference arm: the oracle on the host cores ---------------------------------
def run_reference(args, dist: Dist):
    """The reference algorithm's CPU restatement (the oracle) on all host
    cores.  Its inputs come from oracle-side code only: the seeded generator
    built on its own (oracle/_build/libsynth.so), the oracle's restatement of
    makeDB's packing and of readIndex's clamps; the product library is not
    loaded in this arm."""
    if dist.rank != 0:
        return
    import platform

    from oracle import oracle
    from ngia import CONFIGS  # the workload table (importing it loads no library)

    cfg = dict(CONFIGS[args.workload])
    if args.n_seqs:
        cfg["n_seqs"] = args.n_seqs
    seq, off = oracle.synth(seed=args.seed, **cfg)
    words, rec_off = oracle.pack(cfg["type"], seq, off)
    del seq
    s, w, prec = oracle.clamp(cfg["type"], args.similarity, args.word, 0)
    cores = os.cpu_count() or 1
    times, cands = [], []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        _, _, st = oracle.cluster(words, rec_off, cfg["type"], s, w, prec, threads=0, max_iters=1)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
            cands.append(st["candidates"])
    T = sum(times)
    v = sum(cands) / T
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * T / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u32", "impl": "reference",
           "data": "synthetic (seeded generator with the configuration's shapes)",
           "config": {**workload_desc(args, cfg, words.nbytes), "iters_per_step": 1},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "arch": platform.machine(), "kind": "port",
                            "sample": f"first greedy iteration (representative vs all {len(rec_off):,} sequences) "
                                      f"per step, C/OpenMP restatement of the reference on all host threads"},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "libraries": repo_libraries()}
    print(json.dumps(out), flush=True)


# ---- our arm ------------------------------------------------------------------------
def stage_replay(ctx, ck: str, iters: int, floor: bool = False) -> dict:
    """Resumes the checkpoint taken at the start of the timed region in the
    plain driver with CUDA events around every stage launch on the library
    stream and runs the same `iters` greedy iterations again; returns the
    stage times and the work counters of exactly those iterations, and the
    assignment they end with.  `floor`: first measures the composition
    filter's floor (empty launch, read-only pass) on the unclustered set the
    timed region starts from."""
    import ngia

    ctx.resume(ck, ngia.MODE_PLAIN)
    fl = ctx.filter_floor() if floor else None
    a = ctx.stats()
    ctx.set_profiling(True)
    ctx.step(iters)
    ctx.set_profiling(False)
    cl, ident, b = ctx.end()
    d = {k: (b[k] - a[k]) for k in ("iterations", "candidates", "band_cells", "done_cells", "filter_bytes",
                                    "align_pairs")}
    d["ms_filter"], d["ms_align"] = b["ms_filter"], b["ms_align"]  # the resumed run starts its timers at 0
    for k in ("class_pairs", "class_cells", "class_bytes"):
        d[k] = [y - x for x, y in zip(a[k], b[k])]
    d["class_ms"] = list(b["class_ms"])
    d["floor_us"] = fl
    return d, cl, ident


def align_roofline(rep: dict, db_type: int, int_gops: float, ms_per_step: float, S: int) -> dict:
    """Roofline of the dominant alignment kernel from the replay of the timed
    iterations: in-band cells it computed / its event time, against the INT32
    issue rate x 32 cells / the instructions of one 32-cell update."""
    import ngia

    it = max(1, rep["iterations"])
    k = max(range(len(rep["class_ms"])), key=lambda i: rep["class_ms"][i])
    ms_k = rep["class_ms"][k]
    achieved = rep["class_cells"][k] / (ms_k * 1e-3) / 1e9 if ms_k > 0 else 0.0
    # DNA reads the match word from the representative's match table (AND,
    # add with carry, LOP3); protein builds it from 5 planes (5 LOP3, add, LOP3)
    ops = 3 if db_type == 0 else 7
    peak = int_gops * 32.0 / ops
    names = ngia.class_kernels(db_type)
    return {"bound": "int32", "kernel": names[k], "class": k, "achieved": achieved, "peak": peak, "unit": "Gcell/s",
            "frac": achieved / peak if peak else None,
            "traffic": rep["class_bytes"][k] / it,
            "traffic_kind": "algorithmic bytes per launch (query planes of the pairs the launch aligns; the "
                            "representative's planes are staged once per CTA); one launch per iteration",
            "ms_per_launch": ms_k / it, "launch_ms_per_step": ms_k / it * S, "ms_per_step": ms_per_step,
            "launch_within_step": ms_k / it * S <= ms_per_step, "share_of_step": ms_k / it * S / ms_per_step,
            "peak_source": f"of measured INT32 issue rate {int_gops:.0f} Gop/s (probe, same LOP3/IADD3 mix) x 32 "
                           f"cells / {ops} ops",
            "pairs_per_launch": rep["class_pairs"][k] / it,
            "reference_cells_rate": rep["band_cells"] / (rep["ms_align"] * 1e-3) / 1e9 if rep["ms_align"] else None,
            "replayed_iterations": it, "ms_align_per_iter": rep["ms_align"] / it,
            "class_ms_per_iter": [round(x / it, 4) for x in rep["class_ms"]],
            "class_pairs_per_iter": [round(x / it) for x in rep["class_pairs"]],
            "how": "the timed region starts from a checkpoint; its iterations are replayed from that checkpoint in "
                   "the plain driver with CUDA events around each stage launch (assignments identical)"}


def filter_roofline(rep: dict, peaks: dict) -> dict:
    it = max(1, rep["iterations"])
    ms = rep["ms_filter"]
    gbs = rep["filter_bytes"] / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
    out = {"bound": "hbm", "kernel": "k_prep + k_filter", "achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
           "frac": gbs / peaks["hbm_gbs"], "traffic": rep["filter_bytes"] / it, "peak_source": peaks["source"],
           "traffic_kind": "algorithmic filter bytes per iteration (headers of every candidate, planes of the "
                           "word-tested ones)", "ms_filter_per_iter": ms / it}
    if rep.get("floor_us"):
        launch_us, read_us = rep["floor_us"]
        # at the start of the timed region: the unclustered set is largest there
        out["floor"] = {"empty_launch_us": launch_us, "read_only_us": read_us,
                        "hbm_time_us": 1e6 * (rep["filter_bytes"] / it) / (peaks["hbm_gbs"] * 1e9),
                        "filter_us": 1e3 * ms / it, "filter_over_read_only": (1e3 * ms / it) / read_us if read_us else None,
                        "how": "same grid as the composition filter, same stream, 20 launches each, on the unclustered "
                               "set the timed region starts from: an empty kernel, and one that only reads each "
                               "warp's bitmap words and then the length and counts of every unclustered sequence"}
    return out


def timed_run(args, dist, db, cfg, p, S: int, steps: int, warmup: int, autotune: int, clocks: bool = True):
    """Tuning, warm-up, then `steps` timed steps of S greedy iterations in the
    graph driver (device time on the library stream) from a checkpoint, and
    the stage replay of the same iterations."""
    import numpy as np

    import ngia

    ctx = ngia.Context(db)
    tuning = ctx.autotune(p, autotune) if autotune > 0 else None  # before the timed region
    ctx.begin(p, ngia.MODE_GRAPH)
    for _ in range(warmup):
        ctx.step(S)
    with tempfile.TemporaryDirectory() as td:
        ck = os.path.join(td, "timed.ckpt")
        ctx.save(ck)  # the state the timed region starts from (outside the timing)
        dist.barrier()
        st0 = ctx.stats()
        clk = Clocks(dist.local) if clocks else None
        if clk:
            clk.start()
        t_wall = time.perf_counter()
        dev_ms = 0.0
        for _ in range(steps):
            ctx.step(S)
            dev_ms += ctx.step_ms()
        t_wall = time.perf_counter() - t_wall
        clk_out = clk.stop() if clk else None
        st1 = ctx.stats()
        dist.barrier()
        cl_t, id_t, _ = ctx.end()
        rep, cl_r, id_r = stage_replay(ctx, ck, S * steps, floor=cfg["type"] == 0)
    ctx.close()
    return {"tuning": tuning, "dev_ms": dev_ms, "t_wall": t_wall, "clocks": clk_out,
            "cands": st1["candidates"] - st0["candidates"], "cells": st1["band_cells"] - st0["band_cells"],
            "iters": st1["iterations"] - st0["iterations"], "replay": rep,
            "replay_identical": bool(np.array_equal(cl_t, cl_r) and np.array_equal(id_t, id_r))}


def run_ours(args, dist: Dist):
    import ngia

    ngia.set_device(dist.local)
    db, cfg = make_db(args)
    p = ngia.params_clamp(cfg["type"], args.similarity, args.word, 0)
    S = args.iters_per_step
    int_gops = ngia.measure_int_peak() if dist.rank == 0 else 0.0
    r = timed_run(args, dist, db, cfg, p, S, args.steps, args.warmup, args.autotune)
    T = dist.reduce(r["dev_ms"] / 1e3, "max")
    total_cands = dist.reduce(float(r["cands"]), "sum")
    total_cells = dist.reduce(float(r["cells"]), "sum")
    tuning = r["tuning"]
    # per iteration: prep, filter, next, and per class the thread-per-pair and
    # the warp-per-pair kernel; k_filter_long when short words go first and
    # records exceed 2,048 residues
    launches_per_iter = 3 + 2 * ngia_classes(cfg["type"])
    wo = tuning["word_order"] if tuning else 0
    word_first = wo == 1 or (wo == 0 and (cfg["type"] == 1 or p.similarity >= 0.93))
    if word_first and not p.precise and int(db.words[db.rec_off + 1].max()) > 2048:
        launches_per_iter += 1

    out = None
    if dist.rank == 0:
        peaks = measured_peaks()
        ms_per_step = 1e3 * T / args.steps
        roof = align_roofline(r["replay"], cfg["type"], int_gops, ms_per_step, S)
        froof = filter_roofline(r["replay"], peaks)
        drivers = None if args.skip_drivers or dist.world > 1 else whole_job_drivers(args)
        sweep = similarity_sweep(args, db, cfg) if args.sweep and dist.world == 1 else None
        e2e = None if args.skip_e2e else run_e2e(args, db, p, S)
        cpu = None
        if not args.skip_cpu and dist.world == 1:
            cpu = run_cpu_baseline(args, db, p, cfg)
        secondary = None if args.skip_secondary or dist.world > 1 else run_secondary(args, dist, int_gops, peaks)
        out = {"metric": METRIC, "value": total_cands / T, "unit": UNIT, "n_gpus": dist.world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
               "data": "synthetic (seeded generator with the configuration's shapes)",
               "config": workload_desc(args, cfg, db.words.nbytes),
               "gcups": total_cells / T / 1e9,
               "gcups_note": "reference band cells (func.cu loop bounds) of the pairs aligned, per second",
               "wall_s_timed": r["t_wall"], "iterations_timed": r["iters"],
               "roofline": roof, "filter_roofline": froof, "replay_identical": r["replay_identical"],
               "gpu_launches": launches_per_iter * S * args.steps,
               "drivers_whole_job": drivers, "tuning": tuning, "similarity_sweep": sweep,
               "secondary": secondary, "clocks": r["clocks"], "cpu_baseline": cpu, "e2e": e2e,
               "libraries": repo_libraries()}
    db.close()
    if out is not None:
        print(json.dumps(out), flush=True)


def whole_job_drivers(args) -> dict:
    """The 20,000-sequence DNA configuration clustered to the end by the
    device-side graph driver, the plain host loop and the speculative rounds
    (host clock around ngia_cluster; assignment and scores returned)."""
    import numpy as np

    import ngia

    small_cfg = dict(ngia.CONFIGS["dna_small"])
    sq = ngia.synth(**small_cfg, seed=args.seed)
    sdb = ngia.DB.pack(0, sq, sq.off)
    sq.close()
    sp = ngia.params_clamp(0, args.similarity, args.word, 0)
    times, outs = {}, {}
    with ngia.Context(sdb) as sctx:
        for name, mode in (("graph", ngia.MODE_GRAPH), ("plain", ngia.MODE_PLAIN), ("spec", ngia.MODE_SPEC)):
            sctx.cluster(sp, mode)  # warm-up (graph capture, caches, buffers)
            t0 = time.perf_counter()
            outs[name] = sctx.cluster(sp, mode)
            times[name] = time.perf_counter() - t0
    same = all(np.array_equal(a, b) for name in ("plain", "spec") for a, b in zip(outs["graph"][:2], outs[name][:2]))
    out = {"workload": f"dna_small: {sdb.n:,} DNA sequences (400 ancestors) clustered to the end, "
                       f"s={args.similarity}, w={args.word}",
           "representatives": int(outs["graph"][2]["iterations"]),
           "graph_s": times["graph"], "plain_s": times["plain"], "spec_s": times["spec"],
           "graph_seqs_per_s": sdb.n / times["graph"], "plain_seqs_per_s": sdb.n / times["plain"],
           "spec_seqs_per_s": sdb.n / times["spec"],
           "speedup": times["plain"] / times["graph"], "spec_speedup_vs_plain": times["plain"] / times["spec"],
           "identical": bool(same),
           "forms": "graph: device-side driver, one representative per iteration; plain: host loop, one launch "
                    "sequence per representative; spec: speculative rounds of up to 64 candidate representatives "
                    "once the unclustered set is small",
           "timing": "host clock around ngia_cluster (assignment and scores returned)"}
    sdb.close()
    return out


def similarity_sweep(args, db, cfg) -> list:
    """The same database at the other similarities of its configuration:
    tuned, then timed over a few steps each (graph driver, device time)."""
    import ngia

    S = args.iters_per_step
    out = []
    for sv in (float(x) for x in args.sweep.split(",")):
        sp = ngia.params_clamp(cfg["type"], sv, args.word, 0)
        with ngia.Context(db) as sctx:
            tun = sctx.autotune(sp, args.autotune) if args.autotune > 0 else None
            sctx.begin(sp, ngia.MODE_GRAPH)
            sctx.step(S)
            a0 = sctx.stats()
            ms = 0.0
            for _ in range(args.sweep_steps):
                sctx.step(S)
                ms += sctx.step_ms()
            a1 = sctx.stats()
        out.append({"similarity": sv, "word_length": sp.word_length,
                    "value": (a1["candidates"] - a0["candidates"]) / (ms * 1e-3),
                    "gcups": (a1["band_cells"] - a0["band_cells"]) / (ms * 1e-3) / 1e9,
                    "ms_per_iteration": ms / (args.sweep_steps * S),
                    "iterations": f"{S + 1}-{S * (1 + args.sweep_steps)} of a fresh run",
                    "tuning": {k: tun[k] for k in ("word_order", "refill", "warp_pairs")} if tun else None})
    return out


def run_secondary(args, dist, int_gops: float, peaks: dict) -> dict:
    """Bounded sub-results of the other configurations, in the same run:
    the 200k-protein workload at s=0.9 (value and alignment roofline), the
    serving loop (latency, capacity, oracle replay), the reference's own
    CUDA program beside the drop-in tool on the 20,000-sequence DNA
    configuration (whole program, outputs byte-compared) and a batch of 32
    independent jobs clustered to the end in the pooled, per-job-loop and
    plain forms (assignments compared)."""
    import ngia

    out = {}
    t0 = time.perf_counter()
    try:
        pa = argparse.Namespace(**{**vars(args), "workload": "protein_200k", "similarity": 0.9, "word": 5,
                                   "n_seqs": 0})
        pdb, pcfg = make_db(pa)
        pp = ngia.params_clamp(1, 0.9, 5, 0)
        r = timed_run(pa, dist, pdb, pcfg, pp, args.iters_per_step, 3, 2, args.autotune, clocks=False)
        ms = r["dev_ms"] / 3
        out["protein_200k"] = {"workload": workload_desc(pa, pcfg, pdb.words.nbytes)["workload"],
                               "value": r["cands"] / (r["dev_ms"] * 1e-3), "unit": UNIT, "ms_per_step": ms,
                               "iterations_timed": r["iters"], "gcups": r["cells"] / (r["dev_ms"] * 1e-3) / 1e9,
                               "roofline": align_roofline(r["replay"], 1, int_gops, ms, args.iters_per_step),
                               "filter_roofline": filter_roofline(r["replay"], peaks),
                               "dominant": ("filter" if r["replay"]["ms_filter"] > max(r["replay"]["class_ms"])
                                            else "alignment"),
                               "replay_identical": r["replay_identical"], "tuning": r["tuning"]}
        pdb.close()
    except Exception as e:  # a sub-result never takes the headline down
        out["protein_200k"] = {"error": repr(e)}
    out["protein_200k_s"] = round(time.perf_counter() - t0, 1)
    t0 = time.perf_counter()
    try:
        sa = argparse.Namespace(**{**vars(args), "similarity": 0.9, "word": 5, "cpu_seconds": 10.0,
                                   "warmup": 3})
        out["serve"] = serve_summary(run_serve(sa, dist, emit=False))
    except Exception as e:
        out["serve"] = {"error": repr(e)}
    out["serve_s"] = round(time.perf_counter() - t0, 1)
    t0 = time.perf_counter()
    out["reference_gpu"] = reference_gpu_compare(args)
    out["reference_gpu_s"] = round(time.perf_counter() - t0, 1)
    t0 = time.perf_counter()
    try:  # a bounded batch: 32 jobs of at most 4,000 sequences, clustered to the end
        ba = argparse.Namespace(**{**vars(args), "workload": "batch32", "batch_jobs": 32, "batch_max_seqs": 4000,
                                   "batch_iters": 0, "steps": 1, "warmup": 1})
        r = run_batch(ba, dist, emit=False)
        out["batch"] = {k: r[k] for k in ("value", "unit", "ms_per_step", "gcups", "plain", "loops", "rounds",
                                          "speedup_vs_plain", "speedup_vs_loops", "bit_exact_vs_plain")}
        out["batch"]["workload"] = r["config"]["workload"]
        out["batch"]["form"] = r["config"]["form"] + ", every job clustered to the end"
    except Exception as e:
        out["batch"] = {"error": repr(e)}
    out["batch_s"] = round(time.perf_counter() - t0, 1)
    return out


def serve_summary(r: dict) -> dict:
    keep = ("value", "unit", "latency_ms", "offered_batches_per_s", "achieved_batches_per_s", "capacity",
            "identical_open_loop_and_saturated", "oracle_replay", "gcups", "pairs_aligned")
    return {"workload": r["config"]["workload"], "slots": r["config"]["slots"],
            **{k: r[k] for k in keep if k in r}}


def reference_gpu_compare(args) -> dict:
    """The reference's own CUDA clustering program (built from its sources
    for sm_103a by oracle/ref_cluster.py into baseline/_ref) and the drop-in
    `cluster` tool on the 20,000-sequence DNA configuration: whole-program
    wall time each (database load and result writing included) and a byte
    comparison of cluster.txt / represent.fasta."""
    stage = ROOT / "baseline" / "_ref" / "signalNode" / "src" / "func.cu"
    if not stage.exists():
        return {"unavailable": "the reference's sources are not staged in baseline/_ref/signalNode"}
    try:
        from oracle import ref_cluster

        with tempfile.TemporaryDirectory() as td:
            res = ref_cluster.compare(td, "dna_small", args.similarity, args.word, seed=args.seed, quiet=True)
        ref, ours = res.get("reference", {}), res.get("ours", {})
        if ref.get("seconds") and ours.get("seconds"):
            res["speedup"] = ref["seconds"] / ours["seconds"]
            res["n_seqs_per_s"] = {"reference": res["n_seqs"] / ref["seconds"], "ours": res["n_seqs"] / ours["seconds"]}
        return res
    except Exception as e:
        return {"error": repr(e)}


def ngia_classes(db_type: int) -> int:
    return 7 if db_type == 0 else 5


def run_e2e(args, db, p, S):
    """Through the C ABI with host buffers: every step loads the database from
    pinned host memory into an open context (ngia_reload: H2D copy + header
    build), runs S iterations and returns the assignment and scores (D2H)."""
    import ngia

    ngia.pin_host(db.words)
    ngia.pin_host(db.rec_off)
    try:
        times, cands, dev = [], [], []
        with ngia.Context(db) as ctx:
            for k in range(1 + args.e2e_steps):
                t0 = time.perf_counter()
                ctx.reload(db)
                ctx.begin(p, ngia.MODE_GRAPH)
                ctx.step(S)
                cl, ident, st = ctx.end()
                dt = time.perf_counter() - t0
                if k:
                    times.append(dt)
                    cands.append(st["candidates"])
                    dev.append(ctx.step_ms())
    finally:
        ngia.unpin_host(db.words)
        ngia.unpin_host(db.rec_off)
    T = sum(times)
    return {"value": sum(cands) / T, "unit": UNIT, "h2d_bytes_per_step": int(db.words.nbytes + db.rec_off.nbytes),
            "d2h_bytes_per_step": int(8 * db.n), "steps": len(times),
            "device_ms_per_step": sum(dev) / len(dev), "wall_ms_per_step": 1e3 * T / len(times),
            "iterations": f"greedy iterations 1-{S} of a fresh run every step (the most expensive ones: the "
                          f"longest representatives)",
            "per_step": f"ngia_reload (database from pinned host memory into the open context) + {S} greedy "
                        f"iterations + ngia_cluster_end (assignment and scores to host); host clock"}


def run_cpu_baseline(args, db, p, cfg):
    from oracle import oracle

    t0 = time.perf_counter()
    _, _, st1 = oracle.cluster(db.words, db.rec_off, cfg["type"], p.similarity, p.word_length, p.precise,
                               threads=0, max_iters=1)
    t1 = time.perf_counter() - t0
    n_it = max(1, int(args.cpu_seconds / max(t1, 1e-3)))
    t0 = time.perf_counter()
    _, _, st = oracle.cluster(db.words, db.rec_off, cfg["type"], p.similarity, p.word_length, p.precise,
                              threads=0, max_iters=n_it)
    t = time.perf_counter() - t0
    return {"value": st["candidates"] / t, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"first {n_it} greedy iteration(s) of the same workload ({st['candidates']:,} candidates),"
                      f" C/OpenMP restatement of the reference on all host threads"}


def run_cpu_replicas(args, dist: Dist):
    """Replica plumbing without a GPU (tests): every rank clusters its copy of
    a small workload with the oracle for the timed steps; rank 0 reports the
    summed work over the slowest rank's time, exactly as the GPU arm does."""
    from oracle import oracle
    import ngia

    db, cfg = make_db(args)
    p = ngia.params_clamp(cfg["type"], args.similarity, args.word, 0)
    for _ in range(args.warmup):
        oracle.cluster(db.words, db.rec_off, cfg["type"], p.similarity, p.word_length, p.precise, threads=1,
                       max_iters=args.iters_per_step)
    dist.barrier()
    t0 = time.perf_counter()
    cands = 0
    for _ in range(args.steps):
        _, _, st = oracle.cluster(db.words, db.rec_off, cfg["type"], p.similarity, p.word_length, p.precise,
                                  threads=1, max_iters=args.iters_per_step)
        cands += st["candidates"]
    T = dist.reduce(time.perf_counter() - t0, "max")
    total = dist.reduce(float(cands), "sum")
    dist.barrier()
    if dist.rank == 0:
        print(json.dumps({"metric": METRIC, "value": total / T, "unit": UNIT, "n_gpus": dist.world,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * T / args.steps,
                          "higher_is_better": True, "scaling": "weak", "cpu_only": True,
                          "config": workload_desc(args, cfg)}), flush=True)


# ---- the whole 1M job ------------------------------------------------------------------
def run_whole(args, dist: Dist):
    """The 1,000,000-sequence DNA configuration clustered to the end by one
    driver form (--mode; speculative rounds by default, the form the drop-in
    `cluster` tool runs): sequences / wall time of the whole job.  Along the
    way the run is checkpointed when 0, 25, 50, 75 and 95% of the sequences
    are clustered; from each checkpoint the plain, graph and speculative
    forms then run the next --whole-probe iterations (timed on the host clock,
    assignments compared).  The plain form's whole-job time is estimated by
    scaling each stretch of the measured run by the plain/measured time ratio
    at the checkpoints around it."""
    import numpy as np

    import ngia

    if dist.rank != 0:
        return
    args.workload = "dna_1m"
    db, cfg = make_db(args)
    p = ngia.params_clamp(0, args.similarity, args.word, 0)
    forms = {"plain": ngia.MODE_PLAIN, "graph": ngia.MODE_GRAPH, "spec": ngia.MODE_SPEC}
    main = forms[args.whole_mode]
    marks = [0.0, 0.25, 0.5, 0.75, 0.95]
    ctx = ngia.Context(db)
    tuning = ctx.autotune(p, args.autotune) if args.autotune > 0 else None
    clocks = Clocks(dist.local)
    with tempfile.TemporaryDirectory() as td:
        cks, seg = [], []
        ctx.begin(p, main)
        wall = dev = 0.0
        done, k, curve = False, 0, []
        clocks.start()
        while True:
            cl, _, st = ctx.end()  # progress (outside the timing)
            frac = float((cl >= 0).sum()) / db.n
            while k < len(marks) and frac >= marks[k] and not done:
                path = os.path.join(td, f"m{k}.ckpt")
                ctx.save(path)
                cks.append((marks[k], path, frac, wall, int(st["iterations"])))
                k += 1
            curve.append((int(st["iterations"]), round(frac, 4), round(wall, 2)))
            if done:
                break
            t0 = time.perf_counter()
            done = ctx.step(args.whole_chunk)
            wall += time.perf_counter() - t0
            dev += ctx.step_ms()
        clk = clocks.stop()
        cl_main, id_main, st_main = ctx.end()
        reps = int(st_main["iterations"])
        # the forms side by side from every checkpoint
        probes = []
        for mark, path, frac, w_at, it_at in cks:
            res, outs = {}, {}
            for name, mode in forms.items():
                ctx.resume(path, mode)
                t0 = time.perf_counter()
                ctx.step(args.whole_probe)
                dt = time.perf_counter() - t0
                cl, ident, st = ctx.end()
                outs[name] = (cl, ident)
                res[name] = {"ms_per_iteration": 1e3 * dt / max(1, int(st["iterations"]) - it_at),
                             "iterations": int(st["iterations"]) - it_at}
            same = all(np.array_equal(outs["plain"][0], outs[f][0]) and np.array_equal(outs["plain"][1], outs[f][1])
                       for f in forms)
            probes.append({"mark": mark, "clustered": round(frac, 4), "unclustered": int(round((1 - frac) * db.n)),
                           "representatives_before": it_at, "wall_s_at": round(w_at, 2), "forms": res,
                           "identical": bool(same)})
    ctx.close()
    # plain whole-job estimate: each stretch between checkpoints scaled by the
    # mean plain/measured per-iteration ratio at its two ends
    ratios = [pr["forms"]["plain"]["ms_per_iteration"] / pr["forms"][args.whole_mode]["ms_per_iteration"]
              for pr in probes]
    bounds = [pr["wall_s_at"] for pr in probes] + [wall]
    est = 0.0
    for i in range(len(probes)):
        r = ratios[i] if i + 1 >= len(ratios) else 0.5 * (ratios[i] + ratios[i + 1])
        est += (bounds[i + 1] - bounds[i]) * r
    step = max(1, len(curve) // 60)
    out = {"metric": "seqs/sec (whole clustering job, bit-exact)", "value": db.n / wall, "unit": "seqs/s",
           "n_gpus": 1, "higher_is_better": True, "dtype": "u32",
           "data": "synthetic (seeded generator with the configuration's shapes)",
           "config": {"workload": workload_desc(args, cfg, db.words.nbytes)["workload"], "form": args.whole_mode,
                      "chunk": args.whole_chunk, "probe_iterations": args.whole_probe},
           "wall_s": wall, "device_s": dev / 1e3, "representatives": reps,
           "tuning": tuning, "clocks": clk, "checkpoints": probes,
           "plain_estimate": {"wall_s": est, "seqs_per_s": db.n / est, "ratio_measured_vs_plain": est / wall,
                              "how": "each stretch of the measured run between checkpoints scaled by the plain / "
                                     "measured time per iteration at its ends (mean of the two)"},
           "progress": curve[::step] + ([curve[-1]] if curve[-1] not in curve[::step] else []),
           "libraries": repo_libraries()}
    print(json.dumps(out), flush=True)
    db.close()


# ---- batch workload: many independent jobs -----------------------------------------
def batch_jobs(args):
    """256 seeded jobs: log-uniform 1,000-200,000 sequences each, DNA (lengths
    log-uniform 100-10,000) or protein (the 200k-protein generator), similarity
    drawn from {0.8, 0.9, 0.95}; returns [(db, params, description)]."""
    import math

    import numpy as np

    import ngia

    rng = np.random.default_rng(args.seed)
    jobs = []
    for j in range(args.batch_jobs):
        t = int(rng.integers(0, 2))
        n = int(round(math.exp(rng.uniform(math.log(1e3), math.log(args.batch_max_seqs)))))
        s = float(rng.choice([0.8, 0.9, 0.95]))
        if t == 0:
            cfg = dict(type=0, len_dist=2, n_seqs=n, n_ancestors=max(1, n // 50), len_a=100.0, len_b=10000.0,
                       len_min=100, len_max=10000, subst_max=0.20, indel_frac=0.05, indel_max=3)
        else:
            cfg = dict(type=1, len_dist=1, n_seqs=n, n_ancestors=max(1, n // 25), len_a=380.0, len_b=0.7,
                       len_min=20, len_max=35000, subst_max=0.50, indel_frac=0.05, indel_max=5)
        seqs = ngia.synth(**cfg, seed=args.seed * 100003 + j)
        db = ngia.DB.pack(t, seqs, seqs.off)
        seqs.close()
        jobs.append((db, ngia.params_clamp(t, s, args.word, 0)))
    return jobs


def run_batch(args, dist: Dist, emit: bool = True):
    """Batch arm: every step runs the first S greedy iterations of all jobs
    (--batch-iters; 0 = every job to the end) three ways: the pooled form
    (one graph launch; the jobs of a record type share every launch of a
    round, with cross-job work queues per length bucket), the per-job-loop
    form (one graph launch holding one loop per job) and one job after the
    other with the plain host-loop driver.  All return every job's assignment
    to the host; timed on the host clock around the call (it synchronises);
    the assignments of the three forms are compared."""
    import numpy as np

    import ngia

    ngia.set_device(dist.local)
    S = args.iters_per_step if args.batch_iters < 0 else args.batch_iters
    t0 = time.perf_counter()
    jobs = batch_jobs(args)
    t_gen = time.perf_counter() - t0
    dbs, params = [j[0] for j in jobs], [j[1] for j in jobs]
    n_total = sum(db.n for db in dbs)
    arms = {}
    tuning = None
    with ngia.Batch(dbs) as b:
        if args.batch_autotune > 0:
            t0 = time.perf_counter()
            tun = b.autotune(params, args.batch_autotune)
            tuning = {"iters_per_setting": args.batch_autotune, "seconds": round(time.perf_counter() - t0, 2),
                      "jobs": len(tun), "cached": int(sum(t["cached"] for t in tun)),
                      "policy": ["thread", "cutoff", "tuned"][b.policy()],
                      "ms_per_iter": round(tun[0]["ms_per_iter"], 3),
                      "thread_ms_per_iter": round(tun[0]["default_ms_per_iter"], 3)}
        for mode, name in ((ngia.MODE_POOL, "batch"), (ngia.MODE_GRAPH, "loops"), (ngia.MODE_SPEC, "rounds"),
                           (ngia.MODE_PLAIN, "plain")):
            for _ in range(args.warmup):
                b.run(params, mode, max_iters=S)
            dist.barrier()
            clocks = Clocks(dist.local)
            clocks.start()
            cands = cells = 0
            t = time.perf_counter()
            for _ in range(args.steps):
                cls, ids, st = b.run(params, mode, max_iters=S)
                cands += st["candidates"]
                cells += st["band_cells"]
            T = dist.reduce(time.perf_counter() - t, "max")
            arms[name] = dict(T=T, cands=dist.reduce(float(cands), "sum"), cells=dist.reduce(float(cells), "sum"),
                              clk=clocks.stop(), out=(cls, ids))
    same = all(np.array_equal(a, c) for o in ("plain", "loops", "rounds")
               for a, c in zip(arms["batch"]["out"][0] + arms["batch"]["out"][1],
                               arms[o]["out"][0] + arms[o]["out"][1]))
    for db in dbs:
        db.close()
    if dist.rank != 0:
        return
    bat, pln, lps, rds = arms["batch"], arms["plain"], arms["loops"], arms["rounds"]
    n_dna = sum(1 for db in dbs if db.type == 0)
    out = {"metric": METRIC, "value": bat["cands"] / bat["T"], "unit": UNIT, "n_gpus": dist.world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * bat["T"] / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
           "data": "synthetic (seeded generators with the configuration's shapes)",
           "config": {"workload": f"batch{args.batch_jobs}: {args.batch_jobs} independent jobs "
                                  f"({n_dna} DNA, {args.batch_jobs - n_dna} protein), {n_total:,} sequences, "
                                  f"log-uniform 1,000-{args.batch_max_seqs:,} per job, DNA lengths log-uniform "
                                  f"100-10,000, protein log-normal(median 380, sigma 0.7), s in {{0.8,0.9,0.95}}, "
                                  f"w={args.word} (clamped per job)",
                      "iters_per_step": S, "form": "pooled rounds (NGIA_MODE_POOL)",
                      "step": f"first {S} greedy iterations of every job" if S else "every job clustered to the end",
                      "timing": "host clock around ngia_batch_run (assignments of all jobs returned to host)",
                      "generation_s": round(t_gen, 1)},
           "gcups": bat["cells"] / bat["T"] / 1e9,
           "plain": {"value": pln["cands"] / pln["T"], "ms_per_step": 1e3 * pln["T"] / args.steps,
                     "gcups": pln["cells"] / pln["T"] / 1e9,
                     "form": "jobs one after the other, host loop per representative"},
           "loops": {"value": lps["cands"] / lps["T"], "ms_per_step": 1e3 * lps["T"] / args.steps,
                     "gcups": lps["cells"] / lps["T"] / 1e9,
                     "form": "one graph launch holding one conditional loop per job (NGIA_MODE_GRAPH)"},
           "rounds": {"value": rds["cands"] / rds["T"], "ms_per_step": 1e3 * rds["T"] / args.steps,
                      "gcups": rds["cells"] / rds["T"] / 1e9, "speedup_vs_plain": pln["T"] / rds["T"],
                      "form": "every job's speculative-round driver on host worker threads, one stream per job "
                              "(NGIA_MODE_SPEC)"},
           "speedup_vs_plain": pln["T"] / bat["T"], "speedup_vs_loops": lps["T"] / bat["T"],
           "bit_exact_vs_plain": bool(same), "batch_tuning": tuning,
           "clocks": bat["clk"], "plain_clocks": pln["clk"]}
    if emit:
        print(json.dumps(out), flush=True)
    return out


# ---- serving workload ---------------------------------------------------------------
def serve_workload(args):
    """Resident representatives: the clustering of the 20,000-sequence DNA
    configuration (400 ancestors) at the serving similarity.  Batches: sizes
    log-uniform 1-4,096; each query is a window of log-uniform length
    200-3,000 over descendants of the same ancestors (10% from novel ones),
    joined end to end when the window needs more than one.  Arrivals: a
    Poisson stream of args.serve_rate batches per second."""
    import math

    import numpy as np

    import ngia

    rng = np.random.default_rng(args.seed)
    cfg = dict(ngia.CONFIGS["dna_small"])
    p = ngia.params_clamp(0, args.similarity, args.word, 0)
    seqs = ngia.synth(**cfg, seed=args.seed)
    res_db = ngia.DB.pack(0, seqs, seqs.off)
    seqs.close()
    with ngia.Context(res_db) as ctx:
        cl, _, _ = ctx.cluster(p, ngia.MODE_GRAPH)
    reps = ngia.Records.subset(res_db, np.flatnonzero(cl == np.arange(res_db.n)))
    sizes = [int(round(math.exp(rng.uniform(0.0, math.log(4096))))) for _ in range(args.serve_batches)]
    pool_n = sum(sizes) + 64
    pool = ngia.synth(**{**cfg, "novel_frac": 0.1, "n_seqs": cfg["n_seqs"] + pool_n}, seed=args.seed)
    desc = [pool.bytes(i) for i in range(cfg["n_seqs"], cfg["n_seqs"] + pool_n)]
    pool.close()
    batches, k = [], 0
    for m in sizes:
        qs = []
        for _ in range(m):
            L = int(round(math.exp(rng.uniform(math.log(200), math.log(3000)))))
            buf = desc[k % len(desc)]
            j = k + 1
            while len(buf) < L:
                buf += desc[j % len(desc)]
                j += 1
            k += 1
            a = int(rng.integers(0, len(buf) - L + 1))
            qs.append(buf[a:a + L])
        off = np.zeros(len(qs) + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(q) for q in qs])
        batches.append(ngia.DB.pack(0, b"".join(qs), off))
    gaps = rng.exponential(1.0 / args.serve_rate, size=len(batches))
    return p, res_db, reps, batches, np.cumsum(gaps) - gaps[0]


def run_serve(args, dist: Dist, emit: bool = True):
    """Serving arm: the batches are submitted at their Poisson arrival times
    by one thread while another collects them; latency = arrival to result
    (queueing included), throughput = queries / (first arrival to last
    result).  A bounded sample of the batches is replayed by the oracle."""
    import threading as th

    import numpy as np

    import ngia

    if dist.rank != 0:
        return
    t0 = time.perf_counter()
    p, res_db, reps, batches, arrive = serve_workload(args)
    t_gen = time.perf_counter() - t0
    srv = ngia.Server(reps, p, slots=args.serve_slots, max_batch=4096, max_record_blocks=96)
    for b in batches[:args.warmup]:
        srv.wait(srv.submit(b))
    tickets = [None] * len(batches)
    t_sub = [0.0] * len(batches)
    ready = th.Semaphore(0)

    def submitter(start):
        for i, b in enumerate(batches):
            delay = start + arrive[i] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            t_sub[i] = time.perf_counter()
            tickets[i] = srv.submit(b)
            ready.release()

    clocks = Clocks(dist.local)
    clocks.start()
    start = time.perf_counter() + 0.05
    sub = th.Thread(target=submitter, args=(start,))
    sub.start()
    results, t_done = [None] * len(batches), [0.0] * len(batches)
    for i in range(len(batches)):
        ready.acquire()
        results[i] = srv.wait(tickets[i])
        t_done[i] = t_sub[i] + (results[i][2]["queued_ms"] + results[i][2]["run_ms"]) / 1e3
    sub.join()
    clk = clocks.stop()
    end = max(t_done)
    # capacity: every batch submitted at once (the slots stay busy)
    t_sat = time.perf_counter()
    sat_t = [srv.submit(b) for b in batches]
    sat = [srv.wait(t) for t in sat_t]
    T_sat = time.perf_counter() - t_sat
    same_runs = all(np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) for a, b in zip(results, sat))
    lat = np.array([(t_done[i] - (start + arrive[i])) * 1e3 for i in range(len(batches))])
    run_ms = np.array([r[2]["run_ms"] for r in results])
    n_q = sum(b.n for b in batches)
    T = end - start
    # oracle replay of a bounded sample (the smallest batches first)
    from oracle import oracle
    checked, same, t_chk = 0, True, time.perf_counter()
    for i in np.argsort([b.n for b in batches]):
        if time.perf_counter() - t_chk > args.cpu_seconds:
            break
        b = batches[i]
        rep, ident, _ = oracle.assign(reps.words, reps.rec_off, b.words, b.rec_off, 0, p.similarity, p.word_length,
                                      p.precise)
        same = same and np.array_equal(rep, results[i][0]) and np.array_equal(ident, results[i][1])
        checked += 1
    slots = srv.slots
    srv.close()
    out = {"metric": "seqs/sec (queries served: assigned to resident representatives or clustered, bit-exact)",
           "value": n_q / T, "unit": "query seqs/s", "n_gpus": 1, "steps": len(batches), "warmup": args.warmup,
           "ms_per_step": 1e3 * T / len(batches), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "u32", "data": "synthetic (seeded generators with the configuration's shapes)",
           "config": {"workload": f"serve: resident representatives of the 20,000-sequence DNA configuration at "
                                  f"s={p.similarity:.2f} ({reps.n:,} representatives), {len(batches)} batches of "
                                  f"log-uniform 1-4,096 DNA queries (lengths log-uniform 200-3,000, same ancestors "
                                  f"plus 10% novel), Poisson arrivals at {args.serve_rate:g} batches/s",
                      "slots": slots, "queries": n_q, "generation_s": round(t_gen, 1)},
           "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "mean": float(lat.mean()), "max": float(lat.max()),
                          "run_p50": float(np.percentile(run_ms, 50)), "run_p99": float(np.percentile(run_ms, 99))},
           "offered_batches_per_s": args.serve_rate, "achieved_batches_per_s": len(batches) / T,
           "gcups": sum(r[2]["cells"] for r in results) / T / 1e9,
           "pairs_aligned": int(sum(r[2]["pairs"] for r in results)),
           "capacity": {"queries_per_s": n_q / T_sat, "batches_per_s": len(batches) / T_sat,
                        "gcups": sum(r[2]["cells"] for r in sat) / T_sat / 1e9,
                        "form": "all batches submitted at once"},
           "identical_open_loop_and_saturated": bool(same_runs),
           "oracle_replay": {"batches": checked, "queries": int(sum(batches[i].n for i in
                                                                   np.argsort([b.n for b in batches])[:checked])),
                             "identical": bool(same)},
           "clocks": clk}
    for b in batches:
        b.close()
    res_db.close()
    if emit:
        print(json.dumps(out), flush=True)
    return out


def main():
    args = parse()
    if args.workload.startswith("batch") or args.workload == "serve":
        # one hardware queue per job / slot stream (the default is 8); set
        # before the first CUDA call.  The default run keeps the default, and
        # so do the programs it starts (the reference comparison).
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    dist = Dist()
    try:
        if args.cpu_only:
            run_cpu_replicas(args, dist)
        elif args.impl == "reference":
            run_reference(args, dist)
        elif args.workload.startswith("batch"):
            run_batch(args, dist)
        elif args.workload == "serve":
            run_serve(args, dist)
        elif args.workload == "dna_1m_whole":
            run_whole(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()

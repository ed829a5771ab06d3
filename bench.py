"""Benchmark: BFS GTEPS of the out-of-memory engine at a 25% device budget.

Workload (the configuration the headline metric is quoted on): RMAT scale 24
(16,777,216 vertices), edge factor 16 (268,435,456 directed edges), a=.57
b=.19 c=.19 d=.05, seed 2, self-loops and duplicates kept; static region
capped at 25% of the edge-array bytes (the engine stores edges as a 24-bit
stream, so the cap holds a third of them); the rest are read on demand from
pinned host memory. One step = one BFS from one of 8 seeded
random sources with out-degree > 0 (rotating). SSSP (weights uniform in
[1,63], 25% of the 8-byte edge array) and CC (symmetrised graph, 25%) from the
same configuration are measured after the timed BFS steps and reported beside
it.

value  : sum of reached edges (Graph500 TEPS numerator) / sum of device time
         of the K timed steps (CUDA events on the engine's stream; inputs
         resident: static prefix in HBM, the rest pinned in host memory).
e2e    : the same through the C ABI call a user makes, with the result copied
         into a page-locked host buffer, timed with the host clock (the
         pageable-buffer figure is reported beside it).

python bench.py [--gpus 1] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import faulthandler
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GTEPS at 25% device budget; served queries/s + p99 latency vs plain engine"
T_START = time.time()


def log(msg):
    """Progress of the legs on stderr (stdout carries the one JSON line)."""
    print("[bench %7.1fs] %s" % (time.time() - T_START, msg), file=sys.stderr, flush=True)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=24)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--budget", type=float, default=0.25)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--quick", action="store_true", help="BFS only (skip SSSP/CC legs)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the default thresholds instead of autotuning each graph before its timed runs")
    ap.add_argument("--bfs-tuning", default="",
                    help="huge_degree,segment_edges,dense_div,ctas_per_sm,bu_div: set the headline graph's BFS "
                         "thresholds instead of autotuning them (so a profiler run uses the thresholds of a "
                         "plain run; ncu distorts the autotuner's timings)")
    ap.add_argument("--split", action="store_true",
                    help="profiling aid: time the steps with one launch per region (phase timing)")
    ap.add_argument("--batch", type=int, default=64,
                    help="sources of the multi-source leg (0 skips it)")
    ap.add_argument("--serve", default="20,22,24,26",
                    help="RMAT scales of the resident graphs of the serving leg ('' skips it)")
    ap.add_argument("--serve-queries", type=int, default=10000, help="queries of the serving stream")
    ap.add_argument("--serve-fifo-queries", type=int, default=1000,
                    help="prefix of the stream the plain FIFO engine serves under saturating load")
    ap.add_argument("--serve-budget-gb", type=float, default=12.0)
    ap.add_argument("--serve-sweep", type=int, default=1, help="run the Poisson rate sweep (0 skips it)")
    ap.add_argument("--serve-sweep-queries", type=int, default=1000,
                    help="queries per rate of the batched server's Poisson sweep")
    ap.add_argument("--serve-sweep-fifo-queries", type=int, default=300,
                    help="queries of both servers at half the plain engine's capacity")
    ap.add_argument("--pr-study", type=int, default=0,
                    help="run only the PageRank precision study on an RMAT graph of this scale (seed 3, "
                         "static region 30%% of edge bytes): FP32 scatter vs FP64 GPU run vs the FP64 oracle")
    ap.add_argument("--pr-scale", type=int, default=25,
                    help="RMAT scale of the PageRank leg of the default run (0 skips it)")
    ap.add_argument("--pr-stage-mib", type=lambda x: [int(v) for v in x.split(",") if v], default=[16, 32, 64, 128],
                    help="staging sizes (MiB of the budget, two buffers) of the PageRank study's staged passes")
    ap.add_argument("--batch-sssp", action="store_true", help="add a 64-source batched SSSP leg")
    ap.add_argument("--budget-study", action="store_true",
                    help="BFS GTEPS by static fraction of edge bytes (all in HBM down to all on demand)")
    ap.add_argument("--batch-study", action="store_true",
                    help="only the multi-source legs (BFS and SSSP batches vs single runs), one JSON line")
    ap.add_argument("--link-study", action="store_true",
                    help="host-link rate by run length and the BFS's pattern-limited on-demand ceiling")
    ap.add_argument("--fragment-study", action="store_true",
                    help="edge reads per 4096-edge fragment: what a fragment cache could move off the link")
    ap.add_argument("--gather-study", action="store_true",
                    help="the reference's transfer scheme (host gather + copy per iteration) beside zero-copy reads")
    ap.add_argument("--uvm-study", action="store_true",
                    help="compare BFS on the managed-memory (UVM) engine with the split engine")
    return ap.parse_args()


def pick_sources(ptr, n, seed):
    deg = np.diff(ptr)
    cand = np.nonzero(deg > 0)[0]
    rng = np.random.default_rng(seed)
    return [int(x) for x in rng.choice(cand, size=n, replace=False)]


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          "--query-gpu=" + self.Q, "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                smax.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 4 + k and r[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def load_traffic():
    """Per-launch DRAM bytes of the dominant kernel from a committed ncu summary."""
    try:
        return json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
    except Exception:
        return {}


def reference_arm(args):
    """The reference's iteration scheme (frontier + atomic-min relaxation,
    gpu_kernels.cuh:376-396 / CalculateOpt.cu:60-191) on all host threads."""
    import ascetic_gb300 as A
    import oracle
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    ptr, col = A.rmat_csr(args.scale, args.edge_factor, args.seed)
    srcs = pick_sources(ptr, 8, args.seed)
    threads = os.cpu_count() or 1
    for i in range(args.warmup):
        oracle.relax_mt(0, ptr, col, srcs[i % 8], threads)
    tot_edges, tot_s = 0, 0.0
    for i in range(args.steps):
        s = srcs[i % 8]
        t0 = time.perf_counter()
        out, _ = oracle.relax_mt(0, ptr, col, s, threads)
        dt = time.perf_counter() - t0
        tot_s += dt
        tot_edges += oracle.reached_edges(ptr, out, len(ptr))
    v = tot_edges / tot_s / 1e9
    line = {"metric": METRIC, "value": round(v, 4), "unit": "GTEPS", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * tot_s / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic RMAT",
            "config": workload_config(args),
            "cpu_baseline": {"value": round(v, 4), "unit": "GTEPS", "cores": threads, "kind": "port",
                             "sample": "%d BFS runs of the reference frontier/atomic-min scheme (oracle "
                                       "orc_relax_mt) on %d host threads" % (args.steps, threads)},
            "e2e": {"value": round(v, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def pr_study(args):
    """PageRank precision study: standard PageRank (damping 0.85, uniform start,
    dangling mass spread uniformly, stop at FP64 L1 residual < 1e-9 or 100
    passes) on the in-edge (CSC) arrays of an RMAT graph, FP32 ranks/sums with
    FP64 residual and dangling reductions vs an all-FP64 GPU run vs the FP64
    host oracle; max-abs and L1 error of each."""
    import ascetic_gb300 as A
    import oracle
    t0 = time.time()
    cptr, ccol, od = A.rmat_csr(args.pr_study, 16, 3, transpose=True)
    gen_s = time.time() - t0
    out = {"study": "pagerank precision", "rmat_scale": args.pr_study, "edges": int(cptr[-1]),
           "budget_frac": 0.30, "generate_s": round(gen_s, 1)}
    with A.Graph.from_csr(cptr, ccol, outdeg=od, budget=A.make_budget(frac=0.30)) as g:
        res = {}
        for name, prec in (("fp32", A.F32), ("fp64", A.F64)):
            prm = A.make_params(pr_mode=A.PR_STD, precision=prec)
            g.run("pr", params=prm)
            r, st = g.run("pr", params=prm)
            res[name] = (r.astype(np.float64), st)
        # host-link rate of the on-demand pull: 8 FP32 passes with the static and
        # on-demand regions in separate launches timed apart; the on-demand
        # launch reads every in-edge of the on-demand vertices (tiles of short
        # lists and the segments of long ones) over the host link
        prm = A.make_params(pr_mode=A.PR_STD, precision=A.F32, max_iterations=8,
                            flags=A.RUN_PHASE_TIMING | A.RUN_NO_OUTPUT)
        _, st = g.run("pr", params=prm)
        pull_bytes = float(st["ondemand_bytes"])
        gbs = pull_bytes / (st["ms_ondemand"] * 1e-3) / 1e9 if st["ms_ondemand"] else 0.0
        peak = getattr(args, "link_gbs", 0.0) or 0.0
        out["ondemand_pull_link"] = {
            "kernel": "pr_pull_kernel<float> on-demand region (phase-timed passes)", "bound": "host-link",
            "passes": st["iterations"], "bytes_per_pass": int(pull_bytes / max(1, st["iterations"])),
            "ms_per_pass": round(st["ms_ondemand"] / max(1, st["iterations"]), 3),
            "achieved": round(gbs, 1), "peak": round(peak, 1), "unit": "GB/s",
            "frac": round(gbs / peak, 4) if peak else None,
            "peak_source": "pinned H2D cudaMemcpyAsync measured in this run (asc_link_probe, 1 GiB, best of 3)",
            "ms_static_per_pass": round(st["ms_static"] / max(1, st["iterations"]), 3)}
    t1 = time.perf_counter()
    exact, it, resid = oracle.pr_std_mt(cptr, ccol, od, oracle_threads())
    oracle_s = time.perf_counter() - t1
    for name, (r, st) in res.items():
        out[name] = {"ms": round(st["ms_total"], 2), "passes": st["iterations"], "residual": st["residual"],
                     "max_abs_err_vs_fp64_oracle": float(np.abs(r - exact).max()),
                     "max_rel_err_vs_fp64_oracle": float((np.abs(r - exact) / exact).max()),
                     "l1_err_vs_fp64_oracle": float(np.abs(r - exact).sum()),
                     "ondemand_bytes": st["ondemand_bytes"]}
    # FP32 pass time against the static fraction: every edge in HBM (the pull's
    # random rank gathers alone), the 30% budget, every edge read on demand
    by_budget = {}
    for frac in (1.0, 0.30, 0.0):
        with A.Graph.from_csr(cptr, ccol, outdeg=od, budget=A.make_budget(frac=frac)) as g:
            prm = A.make_params(pr_mode=A.PR_STD, precision=A.F32, flags=A.RUN_NO_OUTPUT)
            g.run("pr", params=prm)
            _, st = g.run("pr", params=prm)
            by_budget[str(frac)] = {"ms_per_pass": round(st["ms_total"] / st["iterations"], 3),
                                    "ondemand_gb_per_pass": round(st["ondemand_bytes"] / st["iterations"] / 1e9, 4),
                                    "ondemand_gbps": round(st["ondemand_bytes"] / (st["ms_total"] * 1e-3) / 1e9, 1)}
    out["fp32_pass_by_budget"] = by_budget
    # staged passes: part of the same 30% budget held as two staging buffers,
    # the on-demand edges copied in chunks every pass (copy engine) while the
    # kernels read the chunk before
    staged = {}
    for mib in args.pr_stage_mib:
        b = A.make_budget(frac=0.30, stage_bytes=mib << 20)
        with A.Graph.from_csr(cptr, ccol, outdeg=od, budget=b) as g:
            prm = A.make_params(pr_mode=A.PR_STD, precision=A.F32)
            g.run("pr", params=prm)
            r, st = g.run("pr", params=prm)
            staged[str(mib)] = {"ms": round(st["ms_total"], 2), "passes": st["iterations"],
                                "ms_per_pass": round(st["ms_total"] / st["iterations"], 3),
                                "static_edge_share": round(g.info.static_edges / g.E, 4),
                                "chunks_per_pass": st["staged_chunks"] // max(1, st["iterations"]),
                                "copied_gb_per_pass": round(st["ondemand_bytes"] / st["iterations"] / 1e9, 4),
                                "copy_gbps": round(st["ondemand_bytes"] / (st["ms_total"] * 1e-3) / 1e9, 1),
                                "max_abs_err_vs_fp64_oracle": float(np.abs(r.astype(np.float64) - exact).max())}
    out["fp32_staged_by_stage_mib"] = staged
    out["fp32_vs_fp64_gpu_max_abs"] = float(np.abs(res["fp32"][0] - res["fp64"][0]).max())
    out["oracle"] = {"passes": it, "residual": resid, "seconds": round(oracle_s, 1), "threads": oracle_threads()}
    out["within_1e-6"] = bool(out["fp32"]["max_abs_err_vs_fp64_oracle"] <= 1e-6)
    print(json.dumps(out), flush=True)


def pagerank_leg(args):
    """The PageRank precision configuration in every default run: RMAT scale
    25 (seed 3), in-edge (CSC) arrays, static region 30% of edge bytes,
    standard PageRank (damping 0.85, stop at FP64 L1 residual < 1e-9 or 100
    passes); the FP32-contribution run and the all-FP64 run against the FP64
    host oracle (max-abs, max relative and L1 error per run), and the FP32 run
    with part of the same budget held as staging buffers for the on-demand
    edges (copied in chunks each pass) beside the in-place reads."""
    import ascetic_gb300 as A
    import oracle
    sc = args.pr_scale
    cptr, ccol, od = A.rmat_csr(sc, 16, 3, transpose=True)
    out = {"rmat_scale": sc, "edges": int(cptr[-1]), "budget_frac": 0.30, "stop": "L1 < 1e-9 or 100 passes"}
    res = {}
    with A.Graph.from_csr(cptr, ccol, outdeg=od, budget=A.make_budget(frac=0.30)) as g:
        out["static_edge_share"] = round(g.info.static_edges / g.E, 4)
        for name, prec in (("fp32", A.F32), ("fp64", A.F64)):
            prm = A.make_params(pr_mode=A.PR_STD, precision=prec)
            g.run("pr", params=prm)
            r, st = g.run("pr", params=prm)
            res[name] = (r.astype(np.float64), st)
        # host-link rate of the on-demand pull: 8 FP32 passes with the static and
        # on-demand regions in separate launches timed apart; the on-demand
        # launch reads every in-edge of the on-demand vertices (tiles of short
        # lists and the segments of long ones) over the host link
        prm = A.make_params(pr_mode=A.PR_STD, precision=A.F32, max_iterations=8,
                            flags=A.RUN_PHASE_TIMING | A.RUN_NO_OUTPUT)
        _, st = g.run("pr", params=prm)
        pull_bytes = float(st["ondemand_bytes"])
        gbs = pull_bytes / (st["ms_ondemand"] * 1e-3) / 1e9 if st["ms_ondemand"] else 0.0
        peak = getattr(args, "link_gbs", 0.0) or 0.0
        out["ondemand_pull_link"] = {
            "kernel": "pr_pull_kernel<float> on-demand region (phase-timed passes)", "bound": "host-link",
            "passes": st["iterations"], "bytes_per_pass": int(pull_bytes / max(1, st["iterations"])),
            "ms_per_pass": round(st["ms_ondemand"] / max(1, st["iterations"]), 3),
            "achieved": round(gbs, 1), "peak": round(peak, 1), "unit": "GB/s",
            "frac": round(gbs / peak, 4) if peak else None,
            "peak_source": "pinned H2D cudaMemcpyAsync measured in this run (asc_link_probe, 1 GiB, best of 3)",
            "ms_static_per_pass": round(st["ms_static"] / max(1, st["iterations"]), 3)}
    stage = args.pr_stage_mib[-1] if args.pr_stage_mib else 128
    with A.Graph.from_csr(cptr, ccol, outdeg=od, budget=A.make_budget(frac=0.30, stage_bytes=stage << 20)) as g:
        prm = A.make_params(pr_mode=A.PR_STD, precision=A.F32)
        g.run("pr", params=prm)
        r, st = g.run("pr", params=prm)
        res["fp32_staged"] = (r.astype(np.float64), st)
        staged_share = round(g.info.static_edges / g.E, 4)
    t1 = time.perf_counter()
    exact, it, resid = oracle.pr_std_mt(cptr, ccol, od, oracle_threads())
    out["oracle"] = {"passes": it, "residual": resid, "seconds": round(time.perf_counter() - t1, 1),
                     "threads": oracle_threads()}
    for name, (r, st) in res.items():
        err = np.abs(r - exact)
        out[name] = {"ms": round(st["ms_total"], 2), "passes": st["iterations"],
                     "ms_per_pass": round(st["ms_total"] / st["iterations"], 3), "residual": st["residual"],
                     "max_abs_err": float(err.max()), "max_rel_err": float((err / exact).max()),
                     "l1_err": float(err.sum()), "ondemand_gb_per_pass":
                         round(st["ondemand_bytes"] / st["iterations"] / 1e9, 4)}
    out["fp32_staged"].update({"stage_mib": stage, "static_edge_share": staged_share,
                               "chunks_per_pass": res["fp32_staged"][1]["staged_chunks"] //
                               max(1, res["fp32_staged"][1]["iterations"])})
    out["within_1e-6"] = all(out[n]["max_abs_err"] <= 1e-6 for n in res)
    return out


def serve_leg(args):
    """Serving: BFS/SSSP/CC/PR queries (mix 50/30/10/10, graph uniform, sources
    uniform over vertices with out-degree > 0) against resident RMAT graphs
    (edge factor 16, seeds 5.., weights uniform in [1,63], static region 25% of
    each graph's edge bytes) under one device budget that covers every device
    allocation. The continuous-batching server against the plain
    one-query-at-a-time FIFO engine on the same GPU: saturating load (the whole
    stream submitted at once; the FIFO engine gets a stated prefix of the same
    stream), then Poisson arrivals at swept rates.

    Every query's values are copied out to host memory. Queries outside the
    checked sample share one host buffer per graph and value type (the copy
    happens, the values are overwritten); the sample (spread over the stream,
    every graph and algorithm) keeps its own buffers, and its BFS/SSSP/CC
    values must equal the plain engine's bit for bit, PageRank within 1e-6."""
    import ascetic_gb300 as A
    scales = [int(x) for x in args.serve.split(",") if x]
    rng = np.random.default_rng(12345)
    graphs, cands = [], []
    t0 = time.time()
    for i, sc in enumerate(scales):
        ptr, adj = A.rmat_csr(sc, 16, 5 + i, weights=(1, 63))
        deg = np.diff(ptr)
        cands.append(np.nonzero(deg > 0)[0])
        graphs.append(A.Graph.from_csr(ptr, adj, budget=A.make_budget(frac=args.budget)))
        del ptr, adj, deg
    # one BFS per graph before any timing: a graph's first BFS builds its
    # in-edges on the host (bottom-up steps), a one-time cost neither server's
    # timed runs should carry
    for gi, g in enumerate(graphs):
        g.run("bfs", int(cands[gi][0]), params=A.make_params(flags=A.RUN_NO_OUTPUT))
    t_gen = time.time() - t0
    log("serving graphs built (%.1f s)" % t_gen)
    std32 = A.make_params(pr_mode=A.PR_STD, precision=A.F32)
    plan = []
    for _ in range(args.serve_queries):
        gi = int(rng.integers(0, len(scales)))
        r = rng.random()
        algo = "bfs" if r < 0.5 else ("sssp" if r < 0.8 else ("cc" if r < 0.9 else "pr"))
        src = int(rng.choice(cands[gi])) if algo in ("bfs", "sssp") else 0
        plan.append((gi, algo, src))
    n_fifo = min(len(plan), args.serve_fifo_queries)
    # checked sample: every k-th query of the FIFO prefix, plus the first query
    # of each (graph, algorithm) pair there
    step = max(1, n_fifo // 48)
    sample = set(range(0, n_fifo, step))
    seen = set()
    for k, (gi, algo, _) in enumerate(plan[:n_fifo]):
        if (gi, algo) not in seen:
            seen.add((gi, algo))
            sample.add(k)
    sinks = {}

    def out_for(k, gi, algo):
        dt = np.float32 if algo == "pr" else np.uint32
        if k in sample:
            return np.empty(graphs[gi].V, dt)
        key = (gi, dt)
        if key not in sinks:
            sinks[key] = np.empty(graphs[gi].V, dt)
        return sinks[key]

    budget = int(args.serve_budget_gb * 1e9)

    def run(mode, rate=None, n=None, keep=False):
        todo = plan if n is None else plan[:n]
        with A.Server(budget_bytes=budget, mode=mode) as srv:
            ids = [srv.add_graph(g) for g in graphs]
            arr = np.cumsum(rng.exponential(1.0 / rate, size=len(todo))) if rate else None
            tick = []
            t_start = time.perf_counter()
            for k, (gi, algo, src) in enumerate(todo):
                if arr is not None:
                    delay = t_start + arr[k] - time.perf_counter()
                    if delay > 0:
                        time.sleep(delay)
                tick.append(srv.submit(ids[gi], algo, src, params=std32 if algo == "pr" else None,
                                       out=out_for(k, gi, algo)))
            kept = {}
            for k, t in enumerate(tick):
                o, _ = srv.wait(t)
                if keep and k in sample:
                    kept[k] = o
            st = srv.stats()
            wall = time.perf_counter() - t_start
        return st, kept, wall

    # warm-up (graph loops, batch state) then saturating load
    run(A.SERVE_BATCHED, n=min(40, len(plan)))
    run(A.SERVE_FIFO, n=min(8, len(plan)))
    log("serving warm-up done")
    sb, kb, wb = run(A.SERVE_BATCHED, keep=True)
    log("batched server: %d queries in %.1f s" % (len(plan), wb))
    sf, kf, wf = run(A.SERVE_FIFO, n=n_fifo, keep=True)
    log("plain FIFO engine: %d queries in %.1f s" % (n_fifo, wf))
    exact, pr_err = True, 0.0
    for k in sorted(sample):
        algo = plan[k][1]
        if algo == "pr":
            pr_err = max(pr_err, float(np.abs(kb[k].astype(np.float64) - kf[k].astype(np.float64)).max()))
        elif not np.array_equal(kb[k], kf[k]):
            exact = False
    del kb, kf
    res = {"graphs_rmat_scales": scales, "queries": len(plan), "mix": "50% BFS / 30% SSSP / 10% CC / 10% PR (FP32)",
           "budget_bytes": budget, "graph_build_s": round(t_gen, 1),
           "batched": {"qps": round(sb["queries_per_s"], 2), "p50_ms": round(sb["p50_ms"], 2),
                       "p99_ms": round(sb["p99_ms"], 2), "device_bytes": sb["device_bytes"],
                       "queries": len(plan), "wall_s": round(wb, 1)},
           "plain_fifo": {"qps": round(sf["queries_per_s"], 2), "p50_ms": round(sf["p50_ms"], 2),
                          "p99_ms": round(sf["p99_ms"], 2), "queries": n_fifo, "wall_s": round(wf, 1),
                          "note": "the first %d queries of the same stream" % n_fifo},
           "qps_speedup": round(sb["queries_per_s"] / sf["queries_per_s"], 2) if sf["queries_per_s"] else None,
           "checked_queries": len(sample), "results_equal_plain_engine": bool(exact),
           "pagerank_max_abs_vs_plain_engine": pr_err, "load": "saturating (all submitted at t=0)"}
    sweep = []
    cap_b, cap_f = sb["queries_per_s"], sf["queries_per_s"]
    if args.serve_sweep:
        for frac in (0.25, 0.5, 0.9):
            rate = frac * cap_b
            b, _, _ = run(A.SERVE_BATCHED, rate=rate, n=min(len(plan), args.serve_sweep_queries))
            sweep.append({"server": "batched", "rate_qps": round(rate, 2), "rate_frac_of_batched_capacity": frac,
                          "p50_ms": round(b["p50_ms"], 2), "p99_ms": round(b["p99_ms"], 2),
                          "queries": min(len(plan), args.serve_sweep_queries)})
        # both servers at a rate the plain engine can sustain (half its capacity)
        rate = 0.5 * cap_f
        n_low = min(len(plan), args.serve_sweep_fifo_queries)
        for name, mode in (("batched", A.SERVE_BATCHED), ("plain_fifo", A.SERVE_FIFO)):
            b, _, _ = run(mode, rate=rate, n=n_low)
            sweep.append({"server": name, "rate_qps": round(rate, 2), "rate_frac_of_fifo_capacity": 0.5,
                          "p50_ms": round(b["p50_ms"], 2), "p99_ms": round(b["p99_ms"], 2), "queries": n_low})
    res["poisson_sweep"] = sweep
    for g in graphs:
        g.close()
    return res


def workload_config(args):
    return {"workload": "BFS on RMAT scale %d ef %d seed %d, 8 seeded sources with out-degree > 0, static region "
                        "capped at %d%% of edge bytes, rest read on demand from pinned host memory"
                        % (args.scale, args.edge_factor, args.seed, round(100 * args.budget)),
            "scale": args.scale, "edge_factor": args.edge_factor, "seed": args.seed, "budget_frac": args.budget,
            "l2": "inputs larger than L2 (edge array %.2f GB as 32-bit words)"
                  % (4.0 * (1 << args.scale) * args.edge_factor / 1e9)}


def link_study(args):
    """How fast can the on-demand reads of this BFS go? The host link's rate
    depends on how long the contiguous runs are (short adjacency lists use
    32-byte sectors and link requests partly). Measures the rate by run length
    (asc_link_probe_runs), takes the on-demand run lengths of every BFS
    iteration from the engine's own levels (consecutive frontier vertices of the
    on-demand region, zero-degree vertices skipped, stored edge width), and
    predicts the pattern-limited on-demand time, against the measured one."""
    import ascetic_gb300 as A
    A.lib()
    ptr, col = A.rmat_csr(args.scale, args.edge_factor, args.seed)
    srcs = pick_sources(ptr, 8, args.seed)
    V = len(ptr) - 1
    sizes = [16, 32, 48, 64, 96, 128, 192, 256, 512, 1024, 4096, 16384]
    curve = {b: A.link_probe_runs(b) for b in sizes}
    dma, smread = A.link_probe(1 << 30, 3)
    xs = np.log(np.array(sizes, dtype=np.float64))
    ys = np.array([curve[b] for b in sizes])

    def rate(run_bytes):
        return np.interp(np.log(np.clip(run_bytes, sizes[0], sizes[-1])), xs, ys)

    deg = np.diff(ptr.astype(np.int64))
    with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=args.budget)) as g:
        S = int(g.info.static_vertices)
        eb = g.info.edge_bits / 8.0
        nz = np.nonzero(deg > 0)[0]
        nz = nz[nz >= S]
        cs = np.concatenate([[0], np.cumsum(deg[nz])])
        pred_s = meas_s = od_bytes = 0.0
        runs_total = 0
        for s in srcs:
            lev, _ = g.run("bfs", s)
            _, st = g.run("bfs", s, params=A.make_params(flags=A.RUN_NO_OUTPUT | A.RUN_PHASE_TIMING))
            meas_s += st["ms_ondemand"] * 1e-3
            lv = lev[nz]
            for it in np.unique(lv):
                if it >= V + 1:
                    continue
                act = (lv == it).astype(np.int8)
                d = np.diff(np.concatenate([[0], act, [0]]))
                starts, ends = np.nonzero(d == 1)[0], np.nonzero(d == -1)[0]
                rb = (cs[ends] - cs[starts]) * eb
                pred_s += float((rb / (rate(rb) * 1e9)).sum())
                od_bytes += float(rb.sum())
                runs_total += len(rb)
    out = {"study": "host-link rate by run length; pattern-limited on-demand ceiling of the BFS",
           "rmat_scale": args.scale, "budget_frac": args.budget, "edge_bits": int(eb * 8),
           "sequential_peak_gbs": {"dma_h2d": round(dma, 1), "sm_reads": round(smread, 1)},
           "runs_gbs_by_bytes": {str(b): round(curve[b], 1) for b in sizes},
           "bfs_runs": len(srcs), "ondemand_bytes_per_bfs": int(od_bytes / len(srcs)),
           "mean_run_bytes": round(od_bytes / max(runs_total, 1), 1),
           "pattern_ceiling_gbs": round(od_bytes / pred_s / 1e9, 1) if pred_s else None,
           "pattern_limited_ms_per_bfs": round(1e3 * pred_s / len(srcs), 3),
           "measured_ondemand_ms_per_bfs": round(1e3 * meas_s / len(srcs), 3),
           "measured_gbs": round(od_bytes / meas_s / 1e9, 1) if meas_s else None}
    if pred_s and meas_s:
        out["fraction_of_pattern_ceiling"] = round(pred_s / meas_s, 3)
        out["fraction_of_sequential_peak"] = round(od_bytes / meas_s / 1e9 / dma, 3)
    print(json.dumps(out), flush=True)


def fragment_study(args):
    """Would a cache of hot edge fragments (the reference's fragment swap) cut
    link bytes? Counts the edges every run reads per 4096-edge fragment
    (RUN_FRAGMENT_COUNTS) for BFS and SSSP from 4 sources each and one CC run on
    the symmetrised graph, then compares the share of reads the static prefix
    serves with the share the best contiguous window of that size and the best
    possible set of the same number of fragments, both chosen with hindsight,
    would serve."""
    import ascetic_gb300 as A
    A.lib()
    prm = A.make_params(flags=A.RUN_NO_OUTPUT | A.RUN_FRAGMENT_COUNTS)
    out = {"study": "edge reads per 4096-edge fragment; static prefix vs best resident set",
           "rmat_scale": args.scale, "budget_frac": args.budget}
    ptr, adj = A.rmat_csr(args.scale, args.edge_factor, args.seed, weights=(1, 63))
    srcs = pick_sources(ptr, 4, args.seed)
    legs = [("bfs", ptr, adj[:, 0].copy(), srcs), ("sssp", ptr, adj, srcs)]
    del adj
    for algo, p_, e_, ss in legs:
        with A.Graph.from_csr(p_, e_, budget=A.make_budget(frac=args.budget)) as g:
            for s_ in ss:
                g.run(algo, s_, params=prm)
            out[algo] = _fragment_shares(g)
    del legs
    sptr, scol = A.rmat_csr(args.scale, args.edge_factor, args.seed, symmetric=True)
    with A.Graph.from_csr(sptr, scol, budget=A.make_budget(frac=args.budget)) as g:
        g.run("cc", params=prm)
        out["cc"] = _fragment_shares(g)
    print(json.dumps(out), flush=True)


def _fragment_shares(g):
    c = g.fragment_counts(reset=True).astype(np.float64)
    k = int(g.info.static_edges) // 4096
    tot = c.sum()
    prefix = c[:k].sum() / tot if tot else 0.0
    best = np.sort(c)[::-1][:k].sum() / tot if tot else 0.0
    # the reference's shifted window (bfs.cu:1909-1935): the best contiguous run
    # of k fragments, wherever it starts
    cs = np.concatenate([[0.0], np.cumsum(c)])
    window = (cs[k:] - cs[:len(cs) - k]).max() / tot if tot and k else 0.0
    return {"edges_read": int(tot), "fragments": len(c), "resident_fragments": k,
            "edge_bits": int(g.info.edge_bits), "static_prefix_share": round(prefix, 4),
            "best_window_share": round(window, 4), "best_resident_share": round(best, 4),
            "link_bytes_saved_at_best": round((best - prefix) / (1 - prefix), 4) if prefix < 1 else 0.0}


def gather_study(args):
    """What the zero-copy reads buy against the reference's own transfer
    scheme on the same GPU and budget: every iteration the on-demand frontier
    goes to the host, host threads gather its edges into page-locked staging,
    one copy moves them over and a kernel expands them (RUN_GATHER_COPY), as
    GraphMeta.cuh:469-578 / CalculateOpt.cu:146-178 do (the reference copies
    from pageable memory, which is slower still)."""
    import ascetic_gb300 as A
    A.lib()
    ptr, col = A.rmat_csr(args.scale, args.edge_factor, args.seed)
    srcs = pick_sources(ptr, 8, args.seed)
    out = {"study": "zero-copy on-demand reads vs host gather + copy per iteration (BFS)",
           "rmat_scale": args.scale, "budget_frac": args.budget, "sources": len(srcs)}
    # with the bit stream (the engine's layout) and with plain 32-bit words (the
    # reference's layout, where the host gather is a plain copy per list)
    for suffix, packing in (("", None), ("_32bit", "0")):
        if packing is not None:
            os.environ["ASC_EDGE_PACKING"] = packing
        with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=args.budget)) as g:
            for name, flags in (("zero_copy", A.RUN_NO_OUTPUT), ("gather_copy", A.RUN_NO_OUTPUT | A.RUN_GATHER_COPY)):
                prm = A.make_params(flags=flags)
                g.run("bfs", srcs[0], params=prm)
                ms, edges, od = 0.0, 0, 0
                for s_ in srcs:
                    _, st = g.run("bfs", s_, params=prm)
                    ms += st["ms_total"]
                    edges += st["reached_edges"]
                    od += st["ondemand_bytes"]
                out[name + suffix] = {"ms_per_bfs": round(ms / len(srcs), 3),
                                      "gteps": round(edges / (ms * 1e-3) / 1e9, 2),
                                      "edge_bits": int(g.info.edge_bits),
                                      "ondemand_edge_bytes_per_bfs": int(od / len(srcs))}
        if packing is not None:
            del os.environ["ASC_EDGE_PACKING"]
    out["zero_copy_speedup"] = round(out["gather_copy"]["ms_per_bfs"] / out["zero_copy"]["ms_per_bfs"], 2)
    out["zero_copy_speedup_32bit"] = round(out["gather_copy_32bit"]["ms_per_bfs"] /
                                           out["zero_copy_32bit"]["ms_per_bfs"], 2)
    # the reference's whole-partition baseline (bfs.cu:6-168): every partition
    # holding a frontier vertex copied whole each iteration. As the reference
    # runs it, the whole budget is the partition buffers (no static region);
    # beside it, a static prefix with 64 MiB of the budget as the buffers.
    budget_bytes = args.budget * 4.0 * int(ptr[-1])
    for name, b in (("partition_copy", A.make_budget(nbytes=budget_bytes, stage_bytes=int(budget_bytes))),
                    ("partition_copy_with_static",
                     A.make_budget(frac=args.budget, stage_bytes=64 << 20))):
        with A.Graph.from_csr(ptr, col, budget=b) as g:
            prm = A.make_params(flags=A.RUN_NO_OUTPUT | A.RUN_PARTITION_COPY)
            g.run("bfs", srcs[0], params=prm)
            ms, edges, moved, copies = 0.0, 0, 0, 0
            for s_ in srcs:
                _, st = g.run("bfs", s_, params=prm)
                ms += st["ms_total"]
                edges += st["reached_edges"]
                moved += st["ondemand_bytes"]
                copies += st["staged_chunks"]
            out[name] = {"ms_per_bfs": round(ms / len(srcs), 3), "gteps": round(edges / (ms * 1e-3) / 1e9, 2),
                         "static_edge_share": round(g.info.static_edges / g.E, 4),
                         "partition_bytes": int(g.info.staging_bytes // 2),
                         "copied_bytes_per_bfs": int(moved / len(srcs)),
                         "partition_copies_per_bfs": round(copies / len(srcs), 1)}
    print(json.dumps(out), flush=True)


def budget_study(args):
    """BFS throughput against the static fraction of the edge bytes, from every
    edge in HBM to every edge read on demand, same graph and sources, thresholds
    autotuned per budget on other sources."""
    import ascetic_gb300 as A
    A.lib()
    ptr, col = A.rmat_csr(args.scale, args.edge_factor, args.seed)
    srcs = pick_sources(ptr, 8, args.seed)
    tune_srcs = pick_sources(ptr, 4, args.seed + 1000)
    out = {"study": "BFS GTEPS by static fraction of edge bytes", "rmat_scale": args.scale, "sources": len(srcs),
           "rows": []}
    for frac in (1.0, 0.75, 0.5, 0.25, 0.1, 0.0):
        with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=frac)) as g:
            if not args.no_tune:
                g.tune("bfs", tune_srcs, cache=False)
            prm = A.make_params(flags=A.RUN_NO_OUTPUT)
            for s_ in srcs[:3]:
                g.run("bfs", s_, params=prm)
            ms, edges, od = 0.0, 0, 0
            for s_ in srcs:
                _, st = g.run("bfs", s_, params=prm)
                ms += st["ms_total"]
                edges += st["reached_edges"]
                od += st["ondemand_bytes"]
            out["rows"].append({"budget_frac": frac, "static_edge_share": round(g.info.static_edges / g.E, 4),
                                "gteps": round(edges / (ms * 1e-3) / 1e9, 2), "ms_per_bfs": round(ms / len(srcs), 3),
                                "ondemand_bytes_per_bfs": int(od / len(srcs)),
                                "ondemand_gbps": round(od / (ms * 1e-3) / 1e9, 1)})
    print(json.dumps(out), flush=True)


def uvm_study(args):
    """The reference's UVM baseline (edges in managed memory, read-mostly, no
    static region) against the split engine at the same graph and sources:
    the managed engine's first BFS pays the page migrations, later ones read
    the GPU-side copies, which sit outside any device budget."""
    import ascetic_gb300 as A
    A.lib()
    ptr, col = A.rmat_csr(args.scale, args.edge_factor, args.seed)
    srcs = pick_sources(ptr, 8, args.seed)
    E = int(ptr[-1])
    out = {"study": "managed-memory (UVM) engine vs split engine", "rmat_scale": args.scale, "edges": E,
           "sources": len(srcs)}
    prm = A.make_params(flags=A.RUN_NO_OUTPUT)

    def leg(budget):
        free0 = A.device_free_bytes()
        with A.Graph.from_csr(ptr, col, budget=budget) as g:
            t = time.perf_counter()
            _, st = g.run("bfs", srcs[0], params=prm)
            first_ms = (time.perf_counter() - t) * 1e3
            ms, edges = [], 0
            for s in srcs:
                _, st = g.run("bfs", s, params=prm)
                ms.append(st["ms_total"])
                edges += st["reached_edges"]
            used = free0 - A.device_free_bytes()
            return {"first_run_ms": round(first_ms, 2), "warm_ms_mean": round(sum(ms) / len(ms), 3),
                    "warm_gteps": round(edges / (sum(ms) * 1e-3) / 1e9, 2),
                    "device_bytes_in_use": int(used), "static_edges": int(g.info.static_edges)}

    out["managed"] = leg(A.make_budget(managed=True))
    out["split_budget_%g" % args.budget] = leg(A.make_budget(frac=args.budget))
    print(json.dumps(out), flush=True)


def replica_setup():
    """Multi-GPU runs are replicas (the path does not shard): under torchrun
    every rank runs the same workload on its own GPU; a gloo group on the host
    gives the barriers and the cross-rank sums/max. Returns (rank, world)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        local = int(os.environ.get("LOCAL_RANK", str(rank)))
        visible = [d for d in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if d]
        # one device per replica process, chosen before the engine library loads
        os.environ["CUDA_VISIBLE_DEVICES"] = visible[local] if local < len(visible) else str(local)
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("gloo")
    return rank, world


def replica_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def replica_reduce(edges, seconds, world):
    """Whole-job totals: edges summed over the replicas, time the slowest one."""
    if world <= 1:
        return edges, seconds
    import torch
    import torch.distributed as dist
    e = torch.tensor([float(edges)], dtype=torch.float64)
    t = torch.tensor([float(seconds)], dtype=torch.float64)
    dist.all_reduce(e, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return e.item(), t.item()


def oracle_threads():
    return os.cpu_count() or 1


def check_rows(mode, ptr, edges, sources, rows):
    """Rows of engine results against the oracle's run of the reference
    frontier scheme on all host threads (oracle.relax_mt: BFS, SSSP and CC have
    one fixpoint each, so any correct schedule gives these exact values).
    Returns (all bit-exact, oracle seconds)."""
    import oracle
    t = time.perf_counter()
    ok = True
    for s_, row in zip(sources, rows):
        exp, _ = oracle.relax_mt(mode, ptr, edges, s_, oracle_threads())
        ok = ok and bool(np.array_equal(np.asarray(row), exp))
    return ok, time.perf_counter() - t


def bfs_32bit_leg(A, ptr, col, srcs, budget, tuning):
    """The same BFS runs with the edges stored as the file's 32-bit words, so the
    25% budget holds exactly 25% of the edges (the reference's layout), beside
    the headline's bit stream (24 bits at scale 24, a third of the edges)."""
    os.environ["ASC_EDGE_PACKING"] = "0"
    try:
        with A.Graph.from_csr(ptr, col, budget=budget) as g:
            if tuning:
                g.set_tuning(**{k: tuning[k] for k in ("huge_degree", "segment_edges", "dense_div", "ctas_per_sm",
                                                        "delta", "bu_div")})
            prm = A.make_params(flags=A.RUN_NO_OUTPUT)
            for s_ in srcs[:3]:
                g.run("bfs", s_, params=prm)
            ms, edges, od = 0.0, 0, 0
            for s_ in srcs:
                _, st = g.run("bfs", s_, params=prm)
                ms += st["ms_total"]
                edges += st["reached_edges"]
                od += st["ondemand_bytes"]
            return {"gteps": round(edges / (ms * 1e-3) / 1e9, 2), "ms_per_bfs": round(ms / len(srcs), 3),
                    "edge_bits": int(g.info.edge_bits), "static_edge_share": round(g.info.static_edges / g.E, 4),
                    "ondemand_bytes_per_bfs": int(od / len(srcs)), "tuning": "the headline graph's"}
    finally:
        del os.environ["ASC_EDGE_PACKING"]


def batch_bfs_leg(A, g, ptr, col, args):
    """One batch of up to 64 BFS sources against the same sources one at a
    time; four rows of that batch (first, last and two between) checked
    against the oracle."""
    bsrc = pick_sources(ptr, args.batch, args.seed + 100)
    # warm-up: the same batch once (its launches are the ones to profile)
    g.run_batch("bfs", bsrc, params=A.make_params(flags=A.RUN_NO_OUTPUT))
    _, bst = g.run_batch("bfs", bsrc, params=A.make_params(flags=A.RUN_NO_OUTPUT))
    seq_ms, seq_edges = 0.0, 0
    for s_ in bsrc:
        _, st = g.run("bfs", s_, params=A.make_params(flags=A.RUN_NO_OUTPUT))
        seq_ms += st["ms_total"]
        seq_edges += st["reached_edges"]
    rows, _ = g.run_batch("bfs", bsrc)
    chk = sorted({0, len(bsrc) // 3, 2 * len(bsrc) // 3, len(bsrc) - 1})
    kept = [rows[i].copy() for i in chk]
    del rows
    exact, oracle_s = check_rows(0, ptr, col, [bsrc[i] for i in chk], kept)
    return {"sources": len(bsrc), "batch_ms": round(bst["ms_total"], 3),
            "sequential_ms": round(seq_ms, 3),
            "speedup": round(seq_ms / bst["ms_total"], 2) if bst["ms_total"] else None,
            "batch_gteps": round(seq_edges / (bst["ms_total"] * 1e-3) / 1e9, 3),
            "ondemand_bytes": bst["ondemand_bytes"], "iterations": bst["iterations"],
            "rows_checked_vs_oracle": chk, "bit_exact": bool(exact), "oracle_s": round(oracle_s, 1)}


def batch_sssp_leg(A, ptr, budget, args):
    """One batch of up to 64 SSSP sources (weights uniform in [1, 63]) against
    the same sources one at a time; rows of the full batch (its many-source
    relaxation path) checked against the oracle when the rows fit in 8 GB of
    host memory, else rows of a 4-source batch."""
    V = len(ptr) - 1
    _, adj = A.rmat_csr(args.scale, args.edge_factor, args.seed, weights=(1, 63))
    with A.Graph.from_csr(ptr, adj, budget=budget) as gw:
        bsrc = pick_sources(ptr, args.batch, args.seed + 200)
        # warm-up: the same batch once (its launches are the ones to profile)
        gw.run_batch("sssp", bsrc, params=A.make_params(flags=A.RUN_NO_OUTPUT))
        _, bst = gw.run_batch("sssp", bsrc, params=A.make_params(flags=A.RUN_NO_OUTPUT))
        seq_ms = 0.0
        for s_ in bsrc:
            _, st = gw.run("sssp", s_, params=A.make_params(flags=A.RUN_NO_OUTPUT))
            seq_ms += st["ms_total"]
        if len(bsrc) * V * 4 <= 8 << 30:
            rows, _ = gw.run_batch("sssp", bsrc)
            chk = sorted({0, len(bsrc) // 3, 2 * len(bsrc) // 3, len(bsrc) - 1})
        else:
            rows, _ = gw.run_batch("sssp", bsrc[:4])
            chk = list(range(min(4, len(bsrc))))
        kept = [rows[i].copy() for i in chk]
        del rows
    exact, oracle_s = check_rows(1, ptr, adj, [bsrc[i] for i in chk], kept)
    return {"sources": len(bsrc), "batch_ms": round(bst["ms_total"], 3),
            "sequential_ms": round(seq_ms, 3),
            "speedup": round(seq_ms / bst["ms_total"], 2) if bst["ms_total"] else None,
            "iterations": bst["iterations"], "edges_processed": bst["edges_processed"],
            "ondemand_bytes": bst["ondemand_bytes"], "rows_checked_vs_oracle": chk,
            "bit_exact": bool(exact), "oracle_s": round(oracle_s, 1)}


def batch_study(args):
    """The multi-source legs alone (no single-source timed steps): a batch of
    up to 64 BFS sources and one of SSSP sources against the same sources one
    at a time, on the default graph and budget."""
    import ascetic_gb300 as A
    A.lib()
    ptr, col = A.rmat_csr(args.scale, args.edge_factor, args.seed)
    budget = A.make_budget(frac=args.budget)
    out = {"study": "multi-source batches vs the same sources one at a time", "rmat_scale": args.scale,
           "budget_frac": args.budget}
    with A.Graph.from_csr(ptr, col, budget=budget) as g:
        out["batch_bfs"] = batch_bfs_leg(A, g, ptr, col, args)
    del col
    out["batch_sssp"] = batch_sssp_leg(A, ptr, budget, args)
    print(json.dumps(out), flush=True)


def main():
    faulthandler.enable()
    args = parse()
    if args.pr_study:
        pr_study(args)
        return
    if args.uvm_study:
        uvm_study(args)
        return
    if args.link_study:
        link_study(args)
        return
    if args.fragment_study:
        fragment_study(args)
        return
    if args.gather_study:
        gather_study(args)
        return
    if args.batch_study:
        batch_study(args)
        return
    if args.budget_study:
        budget_study(args)
        return
    if args.impl == "reference":
        reference_arm(args)
        return
    rank, world = replica_setup()
    import __graft_entry__
    import ascetic_gb300 as A
    if not os.path.exists(A.LIB_PATH):
        __graft_entry__.build()
    A.lib()
    if A.device_count() == 0:
        raise SystemExit("no CUDA device")
    t0 = time.time()
    ptr, col = A.rmat_csr(args.scale, args.edge_factor, args.seed)
    t_gen = time.time() - t0
    srcs = pick_sources(ptr, 8, args.seed)
    V = len(ptr) - 1
    budget = A.make_budget(frac=args.budget)
    g = A.Graph.from_csr(ptr, col, budget=budget)
    info = g.info
    # the autotuner picks the thresholds on sources other than the timed ones
    tune_srcs = pick_sources(ptr, 4, args.seed + 1000)
    t_tune = time.time()
    if args.bfs_tuning:
        hd, sg, dd, cs, bu = (int(x) for x in args.bfs_tuning.split(","))
        g.set_tuning(huge_degree=hd, segment_edges=sg, dense_div=dd, ctas_per_sm=cs, bu_div=bu)
        tuning = g.get_tuning()
    else:
        tuning = None if args.no_tune else g.tune("bfs", tune_srcs, cache=False)
    t_tune = time.time() - t_tune
    nores = A.make_params(flags=A.RUN_NO_OUTPUT)
    for i in range(args.warmup):
        g.run("bfs", srcs[i % 8], params=A.make_params(flags=A.RUN_NO_OUTPUT))
    clocks = Clocks()
    clocks.start()
    time.sleep(0.3)
    tot_edges, tot_ms, launches, od_bytes, iters = 0, 0.0, 0, 0, 0
    replica_barrier(world)
    t_wall = time.perf_counter()
    step_flags = A.RUN_NO_OUTPUT | (A.RUN_PHASE_TIMING if args.split else 0)
    for i in range(args.steps):
        _, st = g.run("bfs", srcs[i % 8], params=A.make_params(flags=step_flags))
        tot_edges += st["reached_edges"]
        tot_ms += st["ms_total"]
        launches += st["kernel_launches"]
        od_bytes += st["ondemand_bytes"]
        iters += st["iterations"]
    t_wall = time.perf_counter() - t_wall
    log("timed BFS steps done: %.1f GTEPS" % (tot_edges / (tot_ms * 1e-3) / 1e9))
    replica_barrier(world)
    clk = clocks.stop()
    job_edges, job_s = replica_reduce(tot_edges, tot_ms * 1e-3, world)
    value = job_edges / job_s / 1e9

    # end to end through the C ABI, the levels copied into a page-locked host
    # buffer (asc_host_alloc) every step; the same with a pageable buffer beside it
    n_e2e = min(args.steps, 8)

    def e2e_leg(out):
        edges, secs, od = 0, 0.0, 0
        for i in range(n_e2e):
            t1 = time.perf_counter()
            _, st = g.run("bfs", srcs[i % 8], out=out)
            secs += time.perf_counter() - t1
            edges += st["reached_edges"]
            od += st["ondemand_bytes"]
        return edges, secs, od

    pinned = A.PinnedArray(V, np.uint32)
    e2e_edges, e2e_s, e2e_od = e2e_leg(pinned.array)
    pinned.close()
    pg_edges, pg_s, _ = e2e_leg(np.empty(V, np.uint32))
    e2e_edges, e2e_s = replica_reduce(e2e_edges, e2e_s, world)
    pg_edges, pg_s = replica_reduce(pg_edges, pg_s, world)
    if rank != 0:
        # the replicas' share ends here: rank 0 adds the single-GPU legs and prints
        g.close()
        replica_barrier(world)
        return
    e2e = {"value": round(e2e_edges / e2e_s / 1e9, 4), "unit": "GTEPS",
           "h2d_bytes_per_step": int(e2e_od / n_e2e) + 4, "d2h_bytes_per_step": 4 * V,
           "result_buffer": "page-locked host memory (asc_host_alloc)",
           "value_pageable_result": round(pg_edges / pg_s / 1e9, 4),
           "note": "h2d = on-demand edge bytes read over the host link per BFS plus the source id"}

    # phase split and roofline of the kernels: top-down expansion of the
    # static and of the on-demand region, and the bottom-up steps, each timed
    # with CUDA events on the engine's stream in phase-timed runs of the same
    # sources (same levels, same step directions)
    ms_s = ms_o = ms_b = 0.0
    ed_s = ed_o = ed_b = vs = vo = vx_b = 0
    for i in range(8):
        _, st = g.run("bfs", srcs[i], params=A.make_params(flags=A.RUN_NO_OUTPUT | A.RUN_PHASE_TIMING))
        ms_s += st["ms_static"]
        ms_o += st["ms_ondemand"]
        ms_b += st["ms_bottom_up"]
        ed_b += st["bottom_up_edges"]
        vx_b += st["bottom_up_vertices"]
        ed_o += st["ondemand_edges"] - st["bottom_up_edges"]
        ed_s += st["edges_processed"] - st["ondemand_edges"]
        vo += st["ondemand_vertices"]
        vs += st["frontier_vertices"] - st["ondemand_vertices"]
    peaks = load_peaks()
    hbm_peak = peaks.get("hbm_gbs") or 6800.0
    # algorithmic bytes: the stored column (edge_bits / 8 B) + 4 B destination
    # value per edge and 16 B per frontier vertex (two offsets, own value, list entry)
    eb = info.edge_bits / 8.0
    alg_s = (eb + 4.0) * ed_s + 16.0 * vs
    hbm_gbs = alg_s / (ms_s * 1e-3) / 1e9 if ms_s else 0.0
    link_bytes = eb * ed_o
    dma_gbs, smread_gbs = A.link_probe(1 << 30, 3)
    args.link_gbs = dma_gbs
    link_gbs = link_bytes / (ms_o * 1e-3) / 1e9 if ms_o else 0.0
    # bottom-up: every unreached vertex reads its first in-edge from HBM
    # (bits(V - 1) per vertex) and probes the frontier bitmap (4 B); those whose
    # head is no parent read further in-edges over the host link
    in_eb = float(np.ceil(np.log2(max(V, 2)))) / 8.0
    bu_bytes = vx_b * (in_eb + 4.0) + in_eb * ed_b
    bu_gbs = bu_bytes / (ms_b * 1e-3) / 1e9 if ms_b else 0.0
    bu_link_gbs = in_eb * ed_b / (ms_b * 1e-3) / 1e9 if ms_b else 0.0
    ms_all = ms_s + ms_o + ms_b
    traffic = load_traffic()
    shares = {"static": ms_s, "on-demand": ms_o, "bottom-up": ms_b}
    dominant = max(shares, key=shares.get)
    link_common = {"peak_source": "pinned H2D cudaMemcpyAsync measured in this run",
                   "peak_method": "asc_link_probe: one 1 GiB page-locked buffer copied host to device with "
                                  "cudaMemcpyAsync, best of 3 (sm_zero_copy_read_peak: the SMs reading the same "
                                  "buffer in place with 16-byte loads, best of 3)",
                   "sm_zero_copy_read_peak": round(smread_gbs, 1)}
    roof_static = {"kernel": "expand_fused_kernel<BFS> static region (top-down)", "bound": "hbm",
                   "achieved": round(hbm_gbs, 1), "peak": hbm_peak, "unit": "GB/s",
                   "frac": round(hbm_gbs / hbm_peak, 4),
                   "traffic": (traffic.get("static") or {}).get("dram_bytes_per_launch"),
                   "traffic_source": "profiles/traffic.json (ncu, DRAM read+write bytes per launch)",
                   "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)",
                   "ms_share": round(ms_s / ms_all, 3) if ms_all else None}
    roof_link = dict({"kernel": "expand_fused_kernel<BFS> on-demand region (top-down)", "bound": "host-link",
                      "achieved": round(link_gbs, 1), "peak": round(dma_gbs, 1), "unit": "GB/s",
                      "frac": round(link_gbs / dma_gbs, 4) if dma_gbs else None,
                      "traffic": (traffic.get("ondemand") or {}).get("dram_bytes_per_launch"),
                      "link_traffic": (traffic.get("ondemand") or {}).get("link_bytes_per_launch"),
                      "traffic_source": "profiles/traffic.json (ncu: DRAM read+write and host-link sector bytes "
                                        "per on-demand launch)",
                      "ms_share": round(ms_o / ms_all, 3) if ms_all else None}, **link_common)
    roof_bu = {"kernel": "bottom_up_kernel (BFS bottom-up steps)", "bound": "hbm",
               "achieved": round(bu_gbs, 1), "peak": hbm_peak, "unit": "GB/s",
               "frac": round(bu_gbs / hbm_peak, 4),
               "traffic": (traffic.get("bottom_up") or {}).get("dram_bytes_per_launch"),
               "link_traffic": (traffic.get("bottom_up") or {}).get("link_bytes_per_launch"),
               "traffic_source": "profiles/traffic.json (ncu, per bottom-up launch)",
               "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)",
               "algorithmic_bytes": "unreached vertices examined x (bits(V-1)/8 head + 4 B frontier probe) + "
                                    "in-edges read from host memory x bits(V-1)/8",
               "vertices_examined_per_bfs": int(vx_b / 8), "in_edges_read_per_bfs": int(ed_b / 8),
               "link_gbs_of_host_in_edges": round(bu_link_gbs, 1),
               "ms_share": round(ms_b / ms_all, 3) if ms_all else None}
    roofline = dict({"static": roof_static, "on-demand": roof_link, "bottom-up": roof_bu}[dominant])
    roofline["dominant"] = dominant

    # parity of the timed workload: the levels of every timed source (run again
    # with output, after the timed region) against the oracle
    parity = {"oracle": "oracle.relax_mt: the reference's frontier/atomic-min scheme on %d host threads "
                        "(BFS, SSSP and CC have one fixpoint each)" % oracle_threads()}
    lv = [g.run("bfs", s_)[0] for s_ in srcs]
    ok, o_s = check_rows(0, ptr, col, srcs, lv)
    del lv
    parity["bfs"] = {"sources": len(srcs), "bit_exact": ok, "oracle_s": round(o_s, 1)}
    log("roofline legs and BFS parity done")

    line = {"metric": METRIC, "value": round(value, 4), "unit": "GTEPS", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(tot_ms / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic RMAT (seeded)",
            "config": dict(workload_config(args), tuning=tuning and {k: tuning[k] for k in (
                "huge_degree", "segment_edges", "dense_div", "ctas_per_sm", "bu_div")}, tuning_s=round(t_tune, 2)),
            "e2e": e2e, "gpu_launches": launches, "clocks": clk,
            "roofline": roofline, "roofline_static_hbm": roof_static, "roofline_ondemand_link": roof_link,
            "roofline_bottom_up_link": roof_bu,
            "graph": {"V": V, "E": int(g.E), "edge_bits": int(info.edge_bits), "static_edges": int(info.static_edges),
                      "static_vertices": int(info.static_vertices), "device_edge_bytes": int(info.device_edge_bytes),
                      "ondemand_bytes_per_bfs": int(od_bytes / args.steps), "iterations_per_bfs": iters / args.steps,
                      "generate_s": round(t_gen, 2)},
            "host_wall_ms_per_step": round(1e3 * t_wall / args.steps, 3)}
    if args.batch:
        line["batch_bfs"] = batch_bfs_leg(A, g, ptr, col, args)
        log("batch BFS leg done")
        parity["batch_bfs_rows"] = {"rows": line["batch_bfs"]["rows_checked_vs_oracle"],
                                    "bit_exact": line["batch_bfs"]["bit_exact"]}
    g.close()
    if not args.quick:
        line["bfs_32bit_edges"] = bfs_32bit_leg(A, ptr, col, srcs, budget, tuning)
        log("32-bit edge BFS leg done")
    if args.batch and args.batch_sssp:
        line["batch_sssp"] = batch_sssp_leg(A, ptr, budget, args)

    if not args.quick:
        log("SSSP and CC legs")
        extra = {}
        _, adj = A.rmat_csr(args.scale, args.edge_factor, args.seed, weights=(1, 63))
        with A.Graph.from_csr(ptr, adj, budget=budget) as gw:
            if not args.no_tune:
                gw.tune("sssp", tune_srcs, cache=False)
            gw.run("sssp", srcs[0], params=A.make_params(flags=A.RUN_NO_OUTPUT))
            e, ms, proc, its = 0, 0.0, 0, 0
            for s in srcs[:4]:
                _, st = gw.run("sssp", s, params=A.make_params(flags=A.RUN_NO_OUTPUT))
                e += st["reached_edges"]
                ms += st["ms_total"]
                proc += st["edges_processed"]
                its += st["iterations"]
            extra["sssp_gteps"] = round(e / (ms * 1e-3) / 1e9, 4)
            extra["sssp_ms"] = round(ms / 4, 3)
            extra["sssp_processed_per_reached_edge"] = round(proc / e, 3) if e else None
            extra["sssp_iterations"] = its / 4
            extra["sssp_tuning"] = gw.get_tuning()
            dist = [gw.run("sssp", s_)[0] for s_ in srcs[:4]]
        ok, o_s = check_rows(1, ptr, adj, srcs[:4], dist)
        parity["sssp"] = {"sources": 4, "bit_exact": ok, "oracle_s": round(o_s, 1)}
        del adj, dist
        sp, sc = A.rmat_csr(args.scale, args.edge_factor, args.seed, symmetric=True)
        with A.Graph.from_csr(sp, sc, budget=budget) as gs:
            if not args.no_tune:
                gs.tune("cc", cache=False)
            extra["cc_tuning"] = None if args.no_tune else gs.get_tuning()
            _, st = gs.run("cc", params=A.make_params(flags=A.RUN_NO_OUTPUT))
            _, st = gs.run("cc", params=A.make_params(flags=A.RUN_NO_OUTPUT))
            extra["cc_ms"] = round(st["ms_total"], 3)
            extra["cc_processed_edges_per_s_G"] = round(st["edges_processed"] / (st["ms_total"] * 1e-3) / 1e9, 4)
            extra["cc_iterations"] = st["iterations"]
            labels = gs.run("cc")[0]
        ok, o_s = check_rows(2, sp, sc, [0], [labels])
        parity["cc"] = {"bit_exact": ok, "oracle_s": round(o_s, 1)}
        del sp, sc, labels
        line["other_algorithms"] = extra

    if args.serve:
        log("serving leg")
        line["serving"] = serve_leg(args)
        log("serving leg done")
    if args.pr_scale and not args.quick:
        line["pagerank"] = pagerank_leg(args)
        log("PageRank leg done")

    if not args.no_cpu:
        import oracle
        t1 = time.perf_counter()
        out = oracle.bfs(ptr, col, srcs[0])
        dt = time.perf_counter() - t1
        re = oracle.reached_edges(ptr, out, V + 1)
        line["cpu_baseline"] = {"value": round(re / dt / 1e9, 4), "unit": "GTEPS", "cores": 1, "kind": "port",
                                "sample": "one serial queue BFS (oracle orc_bfs) from source %d of the same graph, "
                                          "%.2f s" % (srcs[0], dt)}
    parity["all_bit_exact"] = all(v["bit_exact"] for v in parity.values() if isinstance(v, dict))
    line["parity"] = parity
    if world > 1:
        line["config"]["parallelism"] = "%d independent replicas (the path does not shard)" % world
    print(json.dumps(line), flush=True)
    replica_barrier(world)


if __name__ == "__main__":
    main()

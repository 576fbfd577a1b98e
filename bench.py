"""Benchmark of the Brandes hot path on one GB300 (or N replicas).

Workload (default): clustered fast-bc on the 2048x2048 road grid (4,194,304 vertices,
15,937,326 directed edges; generator of fast-bc_gb300/graphs.py, seed 42) with the reference's
own Louvain partition (seeds 1-4, precision 0.01; tests/golden/grid2048_partition.npz) and the
reference's own k-means pivot sets (KMeansPivotSelector, kfrac 0.5; tests/golden/
grid2048_pivots.npz) of the communities measured.  One step is the GPU part of
ClusteredBrandeBC::computeBC for those communities: every community vertex as a source over its
community (intra BC + border vectors; a prepared plan replayed from captured CUDA graphs), then
every pivot of the communities over the full graph weighted by its class cardinality, then the
intra-BC correction.  The pivot sets of all 290 communities are out of the reference's reach
(its k-means costs up to hours per community), so the step covers the stored communities
(--clusters; default all of them).  --workload grid256-clustered runs the whole 256x256 grid
instead (76 communities with borders, 2,579 pivots), every piece of it from the reference's own
run.

Metric: GTEPS = source x edge relaxations per second (sum over communities of n_c * m_c plus
P * m per step), batched FP32-compensated form; the line also carries the plain FP64 form on
the same step (one source per block, FP64 dependency: `plain_fp64`, with the speed-up over it)
and the FP32C result's error against it (`precision_vs_fp64`).  ``value`` uses the device time
of the kernels (CUDA events on the library stream; inputs resident); ``e2e`` the wall time of
the same C-ABI calls with page-locked host buffers (host<->device copies inside).  L2 is flushed
(a 512 MiB write) before every timed step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--prec fp32c|fp64] [--sched batched|plain] [--workload ...]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "fast-bc_gb300"))

METRIC = "BC GTEPS & s/graph: batched FP32-comp vs plain FP64 on one GB300, rel err≤1e-6"
GOLDEN = os.path.join(ROOT, "tests", "golden")


class Clustered:
    """Inputs of a clustered step: the graph, the communities (reference order), their pivots and
    cardinalities, and the configuration record."""

    def __init__(self, el, clusters, pivots, cards, config, borders=None):
        self.el, self.clusters, self.pivots, self.cards = el, clusters, pivots, cards
        self.borders = borders
        rp, col, _ = el.csr()
        kid = np.full(el.n, -1, np.int64)
        for k, vs in enumerate(clusters):
            kid[vs] = k
        src = np.repeat(np.arange(el.n), np.diff(rp))
        intra = (kid[src] >= 0) & (kid[src] == kid[col])
        mc = np.bincount(kid[src][intra], minlength=len(clusters))
        self.cluster_work = float(sum(len(clusters[k]) * mc[k] for k in range(len(clusters))))
        self.npivots = int(sum(p.size for p in pivots))
        self.work = self.cluster_work + float(self.npivots) * el.m
        self.config = dict(config, relaxations_per_step=self.work, cluster_relaxations_per_step=self.cluster_work,
                           clusters=len(clusters), pivots=self.npivots)


def c5_inputs(args) -> Clustered:
    import graphs

    el = graphs.WORKLOADS["grid2048"]()
    cid = np.load(os.path.join(GOLDEN, "grid2048_partition.npz"))["community"].astype(np.int64)
    pz = np.load(os.path.join(GOLDEN, "grid2048_pivots.npz"))
    stored = [int(c) for c in pz["clusters"]]
    pick = stored if args.clusters == "all" else [stored[int(i)] for i in args.clusters.split(",")]
    clusters, pivots, cards = [], [], []
    for c in pick:
        i = stored.index(c)
        clusters.append(np.nonzero(cid == c)[0].astype(np.int32))  # ascending: the reference's order
        p = pz["pivots"][pz["pivot_off"][i]:pz["pivot_off"][i + 1]]
        k = pz["cards"][pz["pivot_off"][i]:pz["pivot_off"][i + 1]].astype(np.float64)
        if args.max_pivots > 0:
            p, k = p[: args.max_pivots], k[: args.max_pivots]
        pivots.append(p.astype(np.int32))
        cards.append(k)
    sizes = [int(v.size) for v in clusters]
    cfg = {"workload": "clustered fast-bc, 2048x2048 road grid (4,194,304 vertices, "
                       f"{el.m:,} edges), communities {pick} ({sizes} vertices) with their pivot sets",
           "graph_seed": 42, "louvain_seeds": [1, 2, 3, 4], "louvain_precision": 0.01, "kfrac": 0.5,
           "partition": "the reference's LouvainGraphPartition (318 communities, 290 with borders)",
           "pivot_sets": "the reference's KMeansPivotSelector on the stored communities"}
    return Clustered(el, clusters, pivots, cards, cfg)


def c2_inputs(args) -> Clustered:
    import graphs

    el = graphs.WORKLOADS["grid256"]()
    z = np.load(os.path.join(GOLDEN, "grid256_clustered.npz"))
    off, cv = z["cluster_off"], z["cluster_vertices"]
    boff, bv = z["border_off"], z["borders"]
    poff, pv, kv = z["pivot_off"], z["pivots"], z["cards"]
    keep = [c for c in range(off.size - 1) if boff[c + 1] > boff[c]]  # clusters with borders
    if args.small:
        keep = keep[:8]
    clusters = [cv[off[c]:off[c + 1]] for c in keep]
    borders = [bv[boff[c]:boff[c + 1]] for c in keep]
    pivots = [pv[poff[c]:poff[c + 1]] for c in keep]
    cards = [kv[poff[c]:poff[c + 1]].astype(np.float64) for c in keep]
    if args.small:  # the profiling case: the first 256 pivots
        left, pv2, kv2 = 256, [], []
        for p, k in zip(pivots, cards):
            pv2.append(p[:left])
            kv2.append(k[:left])
            left -= pv2[-1].size
        pivots, cards = pv2, kv2
    cfg = {"workload": "clustered fast-bc, 256x256 road grid (65,536 vertices, 248,528 edges)",
           "graph_seed": 42, "louvain_seeds": [1, 2, 3, 4], "louvain_precision": 0.01, "kfrac": 0.5,
           "partition": "the reference's own clustered run (tests/golden/grid256_clustered.npz)",
           "pivot_sets": "the reference's own clustered run"}
    return Clustered(el, clusters, pivots, cards, cfg, borders)


def clustered_inputs(args) -> Clustered:
    return c2_inputs(args) if args.workload == "grid256-clustered" else c5_inputs(args)


def cpu_sample(inp: Clustered, threads: int, budget_s: float = 12.0):
    """The oracle (C restatement of the reference path, OpenMP over sources) on a bounded sample
    of the same workload: whole communities (smallest first) for half the budget, then pivots."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    og = oracle.CSR.from_edgelist(inp.el)
    rp, col = og.rp, og.col
    src_of = np.repeat(np.arange(inp.el.n), np.diff(rp))
    work = 0.0
    t0 = time.perf_counter()
    done_c = 0
    acc = np.zeros(inp.el.n)
    for k in sorted(range(len(inp.clusters)), key=lambda k: inp.clusters[k].size):
        vs = inp.clusters[k]
        inside = np.zeros(inp.el.n, bool)
        inside[vs] = True
        if inp.borders is not None:
            bs = inp.borders[k]
        else:
            cross = inside[src_of] != inside[col]
            isb = np.zeros(inp.el.n, bool)
            isb[src_of[cross]] = True
            isb[col[cross]] = True
            bs = np.nonzero(isb & inside)[0].astype(np.int32)
        est = float(vs.size) * vs.size * 4 / 25e6 / max(threads, 1)  # ~25M relaxations/s per core
        if done_c and time.perf_counter() - t0 + est > budget_s / 2:
            break
        oracle.cluster_eval(og, vs, bs, acc, threads=threads)
        rows = np.concatenate([np.arange(rp[v], rp[v + 1]) for v in vs])
        work += float(vs.size) * int(np.sum(inside[col[rows]]))
        done_c += 1
    t1 = time.perf_counter()
    pv = np.concatenate(inp.pivots)
    kv = np.concatenate(inp.cards)
    chunk = max(threads, 1)
    i = 0
    while i < pv.size and (i == 0 or time.perf_counter() - t1 < budget_s / 2):
        oracle.pivot_batch(og, pv[i:i + chunk], kv[i:i + chunk], acc, threads=threads)
        work += float(min(chunk, pv.size - i)) * inp.el.m
        i += chunk
    dt = time.perf_counter() - t0
    return work / dt / 1e9, dt, f"{done_c} of {len(inp.clusters)} communities + {min(i, pv.size)} of {pv.size} pivots"


def peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def precision_block(got, ref):
    big = np.abs(ref) >= 1e-3 * np.max(np.abs(ref))
    return {"max_abs_over_max": float(np.max(np.abs(got - ref)) / np.max(np.abs(ref))),
            "max_rel_large": float(np.max(np.abs(got[big] - ref[big]) / np.abs(ref[big]))),
            "mean_rel_large": float(np.mean(np.abs(got[big] - ref[big]) / np.abs(ref[big]))),
            "reference": "the plain FP64 form on the GPU (parity-tested against the oracle); the clustered "
                         "BC is a cancellation, so entries below 1e-3 of the largest are bounded through "
                         "max_abs_over_max"}


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.p = None
        self.device = device
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(values, dist=None, device="cpu"):
    """The slowest rank's value of each entry (one all-reduce; identity on one process)."""
    if dist is None:
        return [float(v) for v in values]
    import torch

    t = torch.tensor(values, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def replica_gteps(work_per_step, steps, world, seconds):
    """Whole-job throughput of `world` independent replicas that each ran `steps` steps of
    `work_per_step` relaxations, the slowest taking `seconds`."""
    return work_per_step * steps * world / seconds / 1e9


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local



def run_clustered(args):
    """Our arm on a clustered workload (default: the 2048x2048 grid's stored communities)."""
    ws, rank, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import fastbc_gpu as fg

    fg.init(local)
    if args.ws_budget_mb > 0:
        fg.set_option("ws_budget_mb", args.ws_budget_mb)
    prec = fg.FP32C if args.prec == "fp32c" else fg.FP64
    sched = fg.BATCHED if args.sched == "batched" else fg.PLAIN
    inp = clustered_inputs(args)
    el = inp.el
    g = fg.Graph.from_edgelist(el)  # resident for the whole run
    # the step's inputs and outputs live in page-locked host memory (copied every step)
    pinned_keep = []

    def pinned(a):
        a = np.ascontiguousarray(a)
        wide = a.dtype == np.uint64
        t = torch.empty(a.size, dtype=torch.from_numpy(a.view(np.int64) if wide else a).dtype, pin_memory=True)
        pinned_keep.append(t)
        out = t.numpy().view(np.uint64) if wide else t.numpy()
        out[:] = a
        return out

    cs0 = fg.ClusterSet.from_lists(inp.clusters, inp.borders).with_borders(g)
    cs = fg.ClusterSet(pinned(cs0.off), pinned(cs0.vertices), pinned(cs0.boff), pinned(cs0.borders))
    allp = pinned(np.concatenate(inp.pivots).astype(np.int32))
    allc = pinned(np.concatenate(inp.cards).astype(np.float64))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    defaults = {k: fg.get_option(k) for k in ("delta", "chunk_max", "frontier_threads", "wide_threads")}
    tuned = {}
    if sched == fg.BATCHED and not args.no_autotune:
        import autotune

        tuned["clusters"] = autotune.tune_clusters(g, cs, prec)
        tuned["pivots"] = autotune.tune_pivots(g, allp, allc, prec)

    def knobs(phase):
        for k, v in tuned.get(phase, {}).items():
            fg.set_option(k, v)

    # output arrays, reused from step to step as a caller running the sweep repeatedly would
    entry_off = np.zeros(cs.count + 1, np.int64)
    entry_off[1:] = np.cumsum(np.diff(cs.off) * np.diff(cs.boff))
    ent = int(entry_off[-1])
    prev = {"ev": fg.ClusterEval(pinned(np.zeros(g.n)), pinned(np.zeros(ent)), pinned(np.zeros(ent, np.uint64)),
                                 cs, entry_off)}
    bcbuf = pinned(np.zeros(g.n))
    # per vertex: the summed pivot cardinalities of its community (ClusteredBrandesBC.h:158-164
    # subtracts intraBC[v] * card once per pivot of v's community); 0 outside the communities
    mult = np.zeros(g.n)
    for c in range(len(inp.clusters)):
        mult[inp.clusters[c]] = float(np.sum(inp.cards[c]))

    # the batched form sweeps the communities as a prepared plan: subgraphs uploaded once, every
    # step one replay of the captured CUDA graphs (shared-memory and frontier kernels)
    plan, plan_ms = None, None
    if sched == fg.BATCHED:
        knobs("clusters")
        t0 = time.perf_counter()
        plan = fg.ClusterPlan(g, cs, prec)
        plan_ms = (time.perf_counter() - t0) * 1e3

    def step(p, s, tune=True):
        st1, st2 = fg.Stats(), fg.Stats()
        if tune:
            knobs("clusters")
        if plan is not None and (p, s) == (prec, sched):
            ev = plan.run(st1, copy=False)
        else:
            ev = fg.cluster_eval_batch(g, cs, p, s, stats=st1, out=prev["ev"])
        if tune:
            knobs("pivots")
        bcbuf[:] = ev.intra_bc
        bc = fg.dependency_batch(g, allp, allc, p, s, out=bcbuf, stats=st2)
        bc -= ev.intra_bc * mult  # BC[v] -= intraBC[v] * (cards of v's community) in one pass
        return bc, st1, st2

    for _ in range(max(args.warmup, 0)):
        step(prec, sched)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = Clocks(local) if rank == 0 else None
    dev_ms, wall_ms, h2d, d2h, launches = [], [], 0, 0, 0
    kern = {"warp_ms": 0.0, "block_ms": 0.0, "warp_bytes": 0.0, "block_bytes": 0.0}
    phase_ms = [0.0, 0.0]
    bc = None
    sweep_block_units = 0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bc, st1, st2 = step(prec, sched)
        wall_ms.append((time.perf_counter() - t0) * 1e3)
        dev_ms.append(st1.kernel_ms + st2.kernel_ms)
        phase_ms[0] += st1.kernel_ms
        phase_ms[1] += st2.kernel_ms
        sweep_block_units = st1.block_units
        h2d += st1.h2d_bytes + st2.h2d_bytes
        d2h += st1.d2h_bytes + st2.d2h_bytes
        launches += st1.launches + st2.launches
        for k in kern:
            kern[k] += getattr(st1, k) + getattr(st2, k)
    torch.cuda.synchronize()
    clk = clocks.stop() if clocks else None
    ours_bc = bc.copy()
    tot_dev, tot_wall = max_over_ranks([sum(dev_ms) / 1e3, sum(wall_ms) / 1e3], dist, "cuda")
    value = replica_gteps(inp.work, args.steps, ws, tot_dev)
    e2e = replica_gteps(inp.work, args.steps, ws, tot_wall)
    # the plain FP64 form on the same step (one source per block, FP64 dependency), default knobs
    plain, ref_bc = None, None
    if not args.no_plain and (prec, sched) != (fg.FP64, fg.PLAIN):
        for k, v in defaults.items():
            fg.set_option(k, v)
        step(fg.FP64, fg.PLAIN, tune=False)
        pd, pw = [], []
        for _ in range(max(args.plain_steps, 1)):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            pbc, s1, s2 = step(fg.FP64, fg.PLAIN, tune=False)
            pw.append(time.perf_counter() - t0)
            pd.append((s1.kernel_ms + s2.kernel_ms) / 1e3)
        ref_bc = pbc.copy()
        pdev, pwall = max_over_ranks([sum(pd), sum(pw)], dist, "cuda")
        plain = {"value": replica_gteps(inp.work, len(pd), ws, pdev), "unit": "GTEPS",
                 "ms_per_step": pdev / len(pd) * 1e3, "steps": len(pd),
                 "e2e": replica_gteps(inp.work, len(pd), ws, pwall),
                 "speedup": (pdev / len(pd)) / (tot_dev / args.steps),
                 "e2e_speedup": (pwall / len(pd)) / (tot_wall / args.steps),
                 "form": "FBC_PREC_FP64 + FBC_SCHED_PLAIN: one source per thread block, FP64 dependency, "
                         "default knobs"}
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    # dominant kernel: the one with more device time
    dom = "warp" if kern["warp_ms"] >= kern["block_ms"] else "block"
    achieved = kern[f"{dom}_bytes"] / (kern[f"{dom}_ms"] / 1e3) / 1e9 if kern[f"{dom}_ms"] else 0.0
    peak, peak_src = peak_hbm()
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath) and dom == "block" and (prec, sched) == (fg.FP32C, fg.BATCHED):
        with open(tpath) as f:
            tw = json.load(f).get(args.workload)
        if tw:  # the frontier-kernel launches of one step: ncu's DRAM bytes per source x sources
            traffic = tw["pivot_bytes_per_unit"] * len(allp) + tw.get("sweep_block_bytes_per_unit", 0.0) * sweep_block_units
    kname = {"block": "frontier_kernel (batched, block per source group)" if sched == fg.BATCHED
             else "brandes_block_kernel", "warp": "small_seg_kernel (shared memory, warp per source)"}[dom]
    line = {"metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_dev / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32x2+u64" if prec == fg.FP32C else "f64+u64",
            "data": "synthetic (seeded road grid); partition and pivot sets from the reference's own Louvain and "
                    "k-means",
            "config": dict(inp.config, precision=args.prec, schedule=args.sched, autotuned=tuned,
                           l2="flushed (512 MiB write) before every step", parallelism=f"replicas{ws}"),
            "s_per_graph": tot_dev / args.steps,
            "e2e": {"value": e2e, "unit": "GTEPS", "h2d_bytes_per_step": h2d // max(args.steps, 1),
                    "d2h_bytes_per_step": d2h // max(args.steps, 1), "s_per_graph": tot_wall / args.steps},
            "phases_ms_per_step": {"cluster_sweep": phase_ms[0] / args.steps, "pivots": phase_ms[1] / args.steps},
            "cluster_sweep": {"captured": bool(plan.captured) if plan is not None else False,
                              "plan_create_ms": plan_ms,
                              "note": "the sweep runs inside each timed step as one replay of the prepared plan"},
            "gpu_launches": launches,
            "plain_fp64": plain,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "kernel": kname,
                         "peak_source": peak_src,
                         "bytes_model": "40*m + 52*n per (segment, source) unit",
                         "scope": "the frontier-kernel launches of one step (community sweep + pivots): achieved = "
                                  "their algorithmic bytes / their event time; traffic = ncu DRAM bytes per source "
                                  "x sources"},
            "clocks": clk}
    if ref_bc is not None:
        line["precision_vs_fp64"] = precision_block(ours_bc, ref_bc)
    if not args.no_cpu_baseline:
        v, dt, what = cpu_sample(inp, os.cpu_count() or 1, args.ref_budget)
        line["cpu_baseline"] = {"value": v, "unit": "GTEPS", "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": f"{what} in {dt:.1f} s (C restatement of the reference hot path, "
                                          "OpenMP over sources)"}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def run_reference(args):
    """The reference arm: the reference's CPU path (the oracle port of it, OpenMP over sources, all
    host cores) on the same workload, each step a bounded sample; rank 0 only."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    if args.workload not in ("grid2048-clustered", "grid256-clustered"):
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm runs the clustered workloads"}))
        return 0
    inp = clustered_inputs(args)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(inp, threads, budget_s=2.0)
    vals, samples = [], []
    for _ in range(args.steps):
        v, dt, what = cpu_sample(inp, threads, budget_s=args.ref_budget)
        vals.append(v)
        samples.append(what)
    value = float(np.mean(vals))
    line = {"metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": inp.work / (value * 1e9) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded road grid); partition and pivot sets from the reference's own Louvain and "
                    "k-means",
            "config": dict(inp.config, precision="fp64", schedule="cpu", l2="n/a (CPU)",
                           parallelism=f"{threads} host threads"),
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": threads, "kind": "port",
                             "sample": f"per step: {samples[-1]} (bounded sample, ~{args.ref_budget:.0f} s); "
                                       "C restatement of the reference hot path, OpenMP over sources"},
            "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


class Workload:
    """A configuration measured by --workload (default: the clustered 256x256 grid)."""

    name = ""
    config: dict = {}
    work = 0.0

    def setup(self, fg, args):
        raise NotImplementedError

    def step(self, fg, prec, sched):
        """Run one step; returns the list of fbc Stats of its C-ABI calls."""
        raise NotImplementedError

    def cpu_sample(self, threads, budget_s):
        raise NotImplementedError

    def tune(self, fg, prec):
        """Autotune the batched schedule's knobs for this workload; returns the choice."""
        return {}

    def knobs(self, fg, phase):
        for k, v in getattr(self, "tuned", {}).get(phase, {}).items():
            fg.set_option(k, v)



class ExactWorkload(Workload):
    """Exact Brandes over every source of one graph (the precision configuration: 512x512 grid)."""

    def __init__(self, name, key):
        self.name, self.key = name, key

    def setup(self, fg, args):
        import graphs

        self.el = graphs.WORKLOADS[self.key]()
        self.g = fg.Graph.from_edgelist(self.el)
        self.work = float(self.el.n) * self.el.m
        self.config = {"workload": f"exact Brandes, {self.key} road grid ({self.el.n:,} vertices, "
                                   f"{self.el.m:,} edges), every source", "graph_seed": 42,
                       "relaxations_per_step": self.work}

    def step(self, fg, prec, sched):
        st = fg.Stats()
        self.knobs(fg, "exact")
        self.last = fg.exact_bc(self.g, prec, sched, stats=st)
        return [st]

    def tune(self, fg, prec):
        import autotune

        src = np.arange(self.el.n, dtype=np.int32)
        self.tuned = {"exact": autotune.tune_pivots(self.g, src, None, prec, sample=min(4096, self.el.n))}
        return self.tuned

    def cpu_sample(self, threads, budget_s):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        og = oracle.CSR.from_edgelist(self.el)
        k = max(threads, 1) * 4
        src = np.arange(0, self.el.n, max(1, self.el.n // k))[:k].astype(np.int32)
        t0 = time.perf_counter()
        oracle.exact_bc_sources(og, src, threads=threads)
        dt = time.perf_counter() - t0
        return src.size * self.el.m / dt / 1e9, dt, f"{src.size} of {self.el.n} sources"


class MultiGraph(Workload):
    """Batching: 48 random geometric 3-NN graphs, exact Brandes on each, one persistent launch
    (--sequential: 48 separate calls instead)."""

    name = "rgg48-exact"

    def setup(self, fg, args):
        import graphs

        self.els = graphs.rgg_batch(48)
        self.gs = [fg.Graph.from_edgelist(e) for e in self.els]
        self.sequential = args.sequential
        self.work = float(sum(e.n * e.m for e in self.els))
        self.config = {"workload": "48 random geometric 3-NN graphs, n log-uniform in [1024, 65536], exact "
                                   "Brandes on each", "graph_seed": 7, "sequential": bool(args.sequential),
                       "relaxations_per_step": self.work}

    def step(self, fg, prec, sched):
        self.knobs(fg, "graphs")
        if self.sequential:
            out = []
            for g in self.gs:
                st = fg.Stats()
                fg.exact_bc(g, prec, sched, stats=st)
                out.append(st)
            return out
        st = fg.Stats()
        fg.multi_exact_bc(self.gs, prec, sched, stats=st)
        return [st]

    def tune(self, fg, prec):
        """On the largest graph (most of the work): a sample of its sources."""
        import autotune

        i = int(np.argmax([e.n for e in self.els]))
        src = np.arange(self.els[i].n, dtype=np.int32)
        self.tuned = {"graphs": autotune.tune_pivots(self.gs[i], src, None, prec, sample=2048)}
        return self.tuned

    def cpu_sample(self, threads, budget_s):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        t0 = time.perf_counter()
        work = 0.0
        done = 0
        for e in sorted(self.els, key=lambda e: e.n):
            og = oracle.CSR.from_edgelist(e)
            k = max(threads, 1) * 2
            src = np.arange(0, e.n, max(1, e.n // k))[:k].astype(np.int32)
            oracle.exact_bc_sources(og, src, threads=threads)
            work += src.size * e.m
            done += 1
            if time.perf_counter() - t0 > budget_s:
                break
        dt = time.perf_counter() - t0
        return work / dt / 1e9, dt, f"{2 * max(threads, 1)} sources of each of the {done} smallest graphs"



EXTRA_WORKLOADS = {
    "grid512-exact": lambda: ExactWorkload("grid512-exact", "grid512"),
    "grid32-exact": lambda: ExactWorkload("grid32-exact", "grid32"),
    "rgg48-exact": MultiGraph,
}


def run_extra(args):
    """One of the exact / batching configurations (the default bench line is the clustered workload)."""
    import torch

    import fastbc_gpu as fg

    fg.init(0)
    if args.ws_budget_mb > 0:
        fg.set_option("ws_budget_mb", args.ws_budget_mb)
    prec = fg.FP32C if args.prec == "fp32c" else fg.FP64
    sched = fg.BATCHED if args.sched == "batched" else fg.PLAIN
    wl = EXTRA_WORKLOADS[args.workload]()
    wl.setup(fg, args)
    tuned = wl.tune(fg, prec) if sched == fg.BATCHED and not args.no_autotune else {}
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        wl.step(fg, prec, sched)
    dev = wall = 0.0
    launches = 0
    kern = {"warp_ms": 0.0, "block_ms": 0.0, "warp_bytes": 0.0, "block_bytes": 0.0}
    phases = {}
    clocks = Clocks(0)
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sts = wl.step(fg, prec, sched)
        wall += time.perf_counter() - t0
        for i, st in enumerate(sts):
            dev += st.kernel_ms / 1e3
            launches += st.launches
            ph = phases.setdefault(i, [0.0, 0.0])
            ph[0] += st.kernel_ms
            ph[1] += st.relaxations
            for k in kern:
                kern[k] += getattr(st, k)
    clk = clocks.stop()
    dom = "warp" if kern["warp_ms"] >= kern["block_ms"] else "block"
    achieved = kern[f"{dom}_bytes"] / (kern[f"{dom}_ms"] / 1e3) / 1e9 if kern[f"{dom}_ms"] else 0.0
    peak, peak_src = peak_hbm()
    line = {"metric": METRIC, "value": wl.work * args.steps / dev / 1e9, "unit": "GTEPS", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev / args.steps * 1e3,
            "higher_is_better": True, "dtype": "f32x2+u64" if prec == fg.FP32C else "f64+u64",
            "config": dict(wl.config, precision=args.prec, schedule=args.sched, autotuned=tuned),
            "e2e": {"value": wl.work * args.steps / wall / 1e9, "unit": "GTEPS"},
            "gpu_launches": launches,
            "roofline": {"kernel": dom, "achieved": achieved, "unit": "GB/s", "peak": peak,
                         "frac": achieved / peak if peak else None, "peak_source": peak_src},
            "clocks": clk}
    if len(phases) > 1:
        line["phases"] = [{"device_ms_per_step": ms / args.steps, "gteps": rel / ms / 1e6 if ms else None}
                          for ms, rel in (phases[i] for i in sorted(phases))]
    if args.workload in ("grid512-exact", "grid32-exact") and args.prec == "fp32c" and not args.no_precision:
        wl.step(fg, fg.FP64, sched)
        ref = wl.last.copy()
        wl.step(fg, fg.FP32C, sched)
        got = wl.last
        nz = ref != 0
        rel = np.abs(got[nz] - ref[nz]) / np.abs(ref[nz])
        line["precision_vs_fp64"] = {"max_rel": float(rel.max()), "mean_rel": float(rel.mean()),
                                     "reference": "the FP64 form on the GPU (parity-tested against the oracle)"}
    if not args.no_cpu_baseline:
        v, dt, what = wl.cpu_sample(os.cpu_count() or 1, args.ref_budget)
        line["cpu_baseline"] = {"value": v, "unit": "GTEPS", "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": f"{what} in {dt:.1f} s"}
    print(json.dumps(line), flush=True)
    return 0



def run_text_load(args):
    """Edge-list text -> device graph (fbc_graph_from_text) on the 2048x2048 road grid's text
    (15.9M edges, 293 MB; --small: the 512x512 grid).  A step is one call from the text in host
    memory (pageable, as a file read leaves it) to the device CSR and its host mirror."""
    import torch

    import fastbc_gpu as fg
    import graphs

    fg.init(0)
    name = "grid512" if args.small else "grid2048"
    el = graphs.WORKLOADS[name]()
    text = el.text()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        fg.Graph.from_text(text).free()
    clocks = Clocks(0)
    parse_ms = wall = 0.0
    launches = 0
    st = fg.Stats()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g = fg.Graph.from_text(text, stats=st)
        wall += time.perf_counter() - t0
        parse_ms += st.kernel_ms
        launches += st.launches
        g.free()
    ck = clocks.stop()
    peak, peak_src = 6800.0, "fallback"
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak, peak_src = float(json.load(f)["hbm_gbs"]), "measured"
    # algorithmic bytes of the parse: the text read once, (src, dst, weight) written per edge
    alg = len(text) + 16.0 * el.m
    achieved = alg / (parse_ms / args.steps / 1e3) / 1e9
    line = {"metric": "edge-list text load (parse + CSR build), edges per second", "value": el.m * args.steps / wall / 1e6,
            "unit": "M edges/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8 -> i32/f64", "data": f"synthetic ({name} road grid written as text)",
            "config": {"workload": f"text load, {name} road grid ({el.n} vertices, {el.m} edges, "
                                   f"{len(text)} bytes of text)", "l2": "flushed (512 MiB write) before every step"},
            "e2e": {"value": el.m * args.steps / wall / 1e6, "unit": "M edges/s", "h2d_bytes_per_step": st.h2d_bytes,
                    "d2h_bytes_per_step": st.d2h_bytes},
            "parse_device_ms": parse_ms / args.steps, "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": "tx_count + scan + tx_tokens", "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_src,
                         "bytes_model": "text bytes + 16 per edge"},
            "clocks": ck}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import text_oracle

        t0 = time.perf_counter()
        s, d, w = text_oracle.parse_edge_text_c(text)
        text_oracle.csr_from_edges_c(s, d, w)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": el.m / dt / 1e6, "unit": "M edges/s", "cores": 1, "kind": "port",
                                "sample": f"the whole text in {dt:.1f} s (C restatement of the reference "
                                          "parser and addEdge merge, one thread)"}
    print(json.dumps(line), flush=True)
    return 0



def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--prec", default="fp32c", choices=["fp32c", "fp64"])
    ap.add_argument("--sched", default="batched", choices=["batched", "plain"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-budget", type=float, default=12.0)
    ap.add_argument("--workload", default="grid2048-clustered",
                    choices=["grid2048-clustered", "grid256-clustered", "text-load"] + sorted(EXTRA_WORKLOADS))
    ap.add_argument("--clusters", default="all",
                    help="grid2048-clustered: indices into the stored communities (comma-separated) or 'all'")
    ap.add_argument("--max-pivots", type=int, default=0,
                    help="grid2048-clustered: at most this many pivots per community (profiling cases)")
    ap.add_argument("--no-plain", action="store_true", help="clustered: skip the plain FP64 runs")
    ap.add_argument("--plain-steps", type=int, default=2, help="clustered: timed steps of the plain FP64 form")
    ap.add_argument("--sequential", action="store_true", help="rgg48-exact: one call per graph")
    ap.add_argument("--no-autotune", action="store_true",
                    help="batched schedule: keep the default knobs instead of tuning them first")
    ap.add_argument("--small", action="store_true",
                    help="grid256-clustered: 8 communities and 256 pivots (profiling case); "
                         "text-load: the 512x512 grid's text")
    ap.add_argument("--no-precision", action="store_true",
                    help="exact workloads: skip the FP32C-vs-FP64 comparison runs")
    ap.add_argument("--ws-budget-mb", type=int, default=0,
                    help="cap the block kernels' workspace (fewer concurrent sources; profiling cases)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "text-load":
        return run_text_load(args)
    if args.workload in EXTRA_WORKLOADS:
        return run_extra(args)
    return run_clustered(args)


if __name__ == "__main__":
    sys.exit(main())

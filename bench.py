"""Benchmark of the Brandes hot path on one GB300 (or N replicas).

Workload (default): clustered fast-bc on the 256x256 road-like grid (65,536 vertices,
248,528 directed edges; generator of fast-bc_gb300/graphs.py, seed 42), with the partition
and pivot set that the reference's own Louvain (seeds 1-4, precision 0.01) and k-means pivot
selector (kfrac 0.5) produce on it (tests/golden/grid256_clustered.npz).  One step is the
GPU part of ClusteredBrandeBC::computeBC: every cluster vertex as a source over its cluster
(intra BC + border vectors), then every pivot over the full graph weighted by its class
cardinality, then the intra-BC correction.

Metric: GTEPS = source x edge relaxations per second (sum over clusters of n_c * m_c plus
P * m per step).  ``value`` uses the device time of the kernels (CUDA events on the library
stream; inputs resident); ``e2e`` the wall time of the same C-ABI calls with host buffers
(host<->device copies inside).  L2 is flushed (a 512 MiB write) before every timed step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--prec fp32c|fp64] [--sched batched|plain]
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
FIXTURE = os.path.join(ROOT, "tests", "golden", "grid256_clustered.npz")


def load_workload():
    import graphs

    el = graphs.WORKLOADS["grid256"]()
    z = np.load(FIXTURE)
    return el, z


def cluster_lists(z):
    off, cv = z["cluster_off"], z["cluster_vertices"]
    boff, bv = z["border_off"], z["borders"]
    poff, pv, kv = z["pivot_off"], z["pivots"], z["cards"]
    keep = [c for c in range(off.size - 1) if boff[c + 1] > boff[c]]  # clusters with borders
    return off, cv, boff, bv, poff, pv, kv, keep


def work_per_step(el, z, keep=None):
    """Relaxations per step: sum_c n_c*m_c (cluster-induced edges) + P*m."""
    rp, col, _ = el.csr()
    off, cv, boff, bv, poff, pv, kv, keep0 = cluster_lists(z)
    keep = keep0 if keep is None else keep
    cid = np.full(el.n, -1, np.int64)
    for c in range(off.size - 1):
        cid[cv[off[c]:off[c + 1]]] = c
    src = np.repeat(np.arange(el.n), np.diff(rp))
    intra = cid[src] == cid[col]
    mc = np.bincount(cid[src][intra], minlength=off.size - 1)
    nc = np.diff(off)
    return float(sum(nc[c] * mc[c] for c in keep) + pv.size * el.m)


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


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_sample(el, z, threads: int, budget_s: float = 12.0):
    """The oracle (C restatement of the reference path, OpenMP) on a bounded sample of the
    same workload: whole clusters, then pivots, until the time budget is spent."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    og = oracle.CSR.from_edgelist(el)
    off, cv, boff, bv, poff, pv, kv, keep = cluster_lists(z)
    rp, col = og.rp, og.col
    cid = np.full(el.n, -1, np.int64)
    for c in range(off.size - 1):
        cid[cv[off[c]:off[c + 1]]] = c
    work = 0.0
    t0 = time.perf_counter()
    done_c = done_p = 0
    acc = np.zeros(el.n)
    for c in keep:
        vs = cv[off[c]:off[c + 1]]
        oracle.cluster_eval(og, vs, bv[boff[c]:boff[c + 1]], acc, threads=threads)
        mc = int(np.sum(cid[col[np.concatenate([np.arange(rp[v], rp[v + 1]) for v in vs])]] == c))
        work += float(vs.size) * mc
        done_c += 1
        if time.perf_counter() - t0 > budget_s / 2:
            break
    t1 = time.perf_counter()
    chunk = max(threads, 1) * 2
    i = 0
    while i < pv.size and time.perf_counter() - t1 < budget_s / 2:
        oracle.pivot_batch(og, pv[i:i + chunk], kv[i:i + chunk].astype(np.float64), acc, threads=threads)
        work += float(min(chunk, pv.size - i)) * el.m
        i += chunk
    done_p = min(i, pv.size)
    dt = time.perf_counter() - t0
    return work / dt / 1e9, dt, f"{done_c} of {len(keep)} clusters + {done_p} of {pv.size} pivots"


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    el, z = load_workload()
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup):
        cpu_sample(el, z, threads, budget_s=2.0)
    samples = []
    for _ in range(args.steps):
        v, dt, what = cpu_sample(el, z, threads, budget_s=args.ref_budget)
        vals.append(v)
        samples.append(what)
    value = float(np.mean(vals))
    work = work_per_step(el, z)
    line = {"metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": work / (value * 1e9) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded road grid; reference partition and pivots)",
            "config": {"workload": "clustered fast-bc, 256x256 road grid (65,536 vertices)",
                       "graph_seed": 42, "louvain_seeds": [1, 2, 3, 4], "kfrac": 0.5,
                       "l2": "n/a (CPU)"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": threads, "kind": "port",
                             "sample": f"per step: {samples[-1]} (bounded sample, ~{args.ref_budget:.0f} s); "
                                       "C restatement of the reference hot path, OpenMP over sources"},
            "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
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
    ap.add_argument("--small", action="store_true",
                    help="profiling case: 8 clusters and 256 pivots of the same workload")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    ws, rank, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import fastbc_gpu as fg

    fg.init(local)
    prec = fg.FP32C if args.prec == "fp32c" else fg.FP64
    sched = fg.BATCHED if args.sched == "batched" else fg.PLAIN
    el, z = load_workload()
    off, cv, boff, bv, poff, pv, kv, keep = cluster_lists(z)
    if args.small:
        keep = keep[:8]
        z = dict(z)
        z["pivots"], z["cards"] = pv[:256], kv[:256]
        z["pivot_off"] = np.minimum(poff, 256)
        poff, pv, kv = z["pivot_off"], z["pivots"], z["cards"]
    clusters = [cv[off[c]:off[c + 1]] for c in keep]
    borders = [bv[boff[c]:boff[c + 1]] for c in keep]
    pivots = [pv[poff[c]:poff[c + 1]] for c in range(off.size - 1)]
    cards = [kv[poff[c]:poff[c + 1]] for c in range(off.size - 1)]
    cs = fg.ClusterSet.from_lists(clusters, borders)
    g = fg.Graph.from_edgelist(el)  # resident for the whole run
    allp = np.concatenate(pivots).astype(np.int32)
    allc = np.concatenate(cards).astype(np.float64)
    work = work_per_step(el, z, keep)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step():
        st1, st2 = fg.Stats(), fg.Stats()
        ev = fg.cluster_eval_batch(g, cs, prec, sched, stats=st1)
        bc = fg.dependency_batch(g, allp, allc, prec, sched, out=ev.intra_bc.copy(), stats=st2)
        for c in range(len(clusters)):
            tot = float(np.sum(cards[keep[c]]))
            if tot:
                bc[clusters[c]] -= ev.intra_bc[clusters[c]] * tot
        return bc, st1, st2

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = Clocks(local) if rank == 0 else None
    dev_ms, wall_ms, h2d, d2h, launches = [], [], 0, 0, 0
    kern = {"warp_ms": 0.0, "block_ms": 0.0, "warp_bytes": 0.0, "block_bytes": 0.0}
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bc, st1, st2 = step()
        wall_ms.append((time.perf_counter() - t0) * 1e3)
        dev_ms.append(st1.kernel_ms + st2.kernel_ms)
        h2d += st1.h2d_bytes + st2.h2d_bytes
        d2h += st1.d2h_bytes + st2.d2h_bytes
        launches += st1.launches + st2.launches
        for k in kern:
            kern[k] += getattr(st1, k) + getattr(st2, k)
    torch.cuda.synchronize()
    clk = clocks.stop() if clocks else None
    tot_dev = sum(dev_ms) / 1e3
    tot_wall = sum(wall_ms) / 1e3
    if dist:
        t = torch.tensor([tot_dev, tot_wall], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_dev, tot_wall = float(t[0]), float(t[1])
    value = work * args.steps * ws / tot_dev / 1e9
    e2e = work * args.steps * ws / tot_wall / 1e9
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    # dominant kernel: the one with more device time
    dom = "warp" if kern["warp_ms"] >= kern["block_ms"] else "block"
    achieved = kern[f"{dom}_bytes"] / (kern[f"{dom}_ms"] / 1e3) / 1e9 if kern[f"{dom}_ms"] else 0.0
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak, peak_src = float(json.load(f)["hbm_gbs"]), "measured"
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get(f"{dom}_{args.prec}_{args.sched}")
    line = {"metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_dev / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32x2+u64" if prec == fg.FP32C else "f64+u64",
            "data": "synthetic (seeded road grid; partition and pivots from the reference's Louvain + k-means)",
            "config": {"workload": "clustered fast-bc, 256x256 road grid (65,536 vertices, 248,528 edges)",
                       "graph_seed": 42, "louvain_seeds": [1, 2, 3, 4], "louvain_precision": 0.01,
                       "kfrac": 0.5, "clusters": len(keep), "pivots": int(allp.size),
                       "relaxations_per_step": work, "precision": args.prec, "schedule": args.sched,
                       "l2": "flushed (512 MiB write) before every step", "parallelism": f"replicas{ws}"},
            "s_per_graph": tot_dev / args.steps,
            "e2e": {"value": e2e, "unit": "GTEPS", "h2d_bytes_per_step": h2d // args.steps,
                    "d2h_bytes_per_step": d2h // args.steps, "s_per_graph": tot_wall / args.steps},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "kernel": dom,
                         "peak_source": peak_src,
                         "bytes_model": "40*m + 52*n per (segment, source) unit"},
            "clocks": clk}
    if not args.no_cpu_baseline:
        v, dt, what = cpu_sample(el, z, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": v, "unit": "GTEPS", "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": f"{what} in {dt:.1f} s (C restatement of the reference hot path, "
                                          "OpenMP over sources)"}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Autotuner for the batched schedule's knobs.

Picks, per workload, the bucket width of the near-far distance pass (``delta``), the block
size of the large-segment kernel (``frontier_threads``) and the number of sources per work
item of the shared-memory kernel (``chunk_max``) by timing candidates on a sample of the
workload's units with the library's own CUDA events (``Stats.kernel_ms``).  Results only
change speed, never values: every candidate computes the same distances, path counts and
dependencies (the dependency sum is taken in adjacency order whatever the schedule).

    choice = autotune.tune_pivots(graph, sources, cards, fg.FP32C)      # applies and returns it
    choice = autotune.tune_clusters(graph, cluster_set, fg.FP32C)
"""
from __future__ import annotations

import itertools

import numpy as np

import fastbc_gpu as fg


def _time(f, reps: int = 3) -> float:
    # the least of a few runs: candidates a percent or two apart are otherwise picked by noise
    best = float("inf")
    for _ in range(reps):
        st = fg.Stats()
        f(st)
        best = min(best, st.kernel_ms)
    return best


def _mean_weight(g: fg.Graph) -> float:
    _, _, w = g.csr()
    return float(np.mean(w)) if w.size else 1.0


def _apply(choice: dict) -> dict:
    for k, v in choice.items():
        fg.set_option(k, int(v))
    return choice


def tune_pivots(g: fg.Graph, sources, cards=None, precision: int = fg.FP32C, sample: int = 4096,
                deltas=(2, 4, 8), threads=(64, 96, 128, 512)) -> dict:
    """Whole-graph sources (pivots, exact mode): delta (as multiples of the mean weight) and
    the frontier kernel's block size (for graphs of wide_n or more vertices, which run one
    source per SM, the wide block size, 512 or 1024 threads, and wider buckets).  Up to `sample`
    sources the whole list is timed, so the number of waves over the concurrent slots (which the
    block size sets) is the real one."""
    if g.n >= fg.get_option("wide_n"):
        return _tune_wide(g, sources, cards, precision, sample)
    src = np.asarray(sources, np.int32)
    idx = np.linspace(0, src.size - 1, min(sample, src.size)).astype(np.int64)
    s = src[idx]
    c = None if cards is None else np.asarray(cards, np.float64)[idx]
    mw = _mean_weight(g)
    best, arg = float("inf"), None
    for dm, bt in itertools.product(deltas, threads):
        choice = {"delta": max(1, int(round(dm * mw))), "frontier_threads": bt}
        _apply(choice)
        t = _time(lambda st: fg.dependency_batch(g, s, c, precision, fg.BATCHED, stats=st))
        if t < best:
            best, arg = t, choice
    return _apply(arg)


def _tune_wide(g: fg.Graph, sources, cards, precision: int, sample: int,
               deltas=(4, 8, 16), threads=(512, 1024)) -> dict:
    src = np.asarray(sources, np.int32)
    idx = np.linspace(0, src.size - 1, min(sample, src.size)).astype(np.int64)
    s = src[idx]
    c = None if cards is None else np.asarray(cards, np.float64)[idx]
    mw = _mean_weight(g)
    best, arg = float("inf"), None
    for dm, bt in itertools.product(deltas, threads):
        choice = {"delta": max(1, int(round(dm * mw))), "wide_threads": bt}
        _apply(choice)
        t = _time(lambda st: fg.dependency_batch(g, s, c, precision, fg.BATCHED, stats=st), reps=2)
        if t < best:
            best, arg = t, choice
    return _apply(arg)


def tune_clusters(g: fg.Graph, cs: fg.ClusterSet, precision: int = fg.FP32C, sample: int = 16,
                  deltas=(2, 4, 8), chunks=(128, 512), threads=(128,)) -> dict:
    """Cluster sources: delta, the shared-memory kernel's chunk size and (for clusters too large
    for shared memory) the frontier kernel's block size, on a sample of the clusters (every k-th,
    keeping the size mix)."""
    cs = cs.with_borders(g)
    k = max(1, cs.count // sample)
    pick = list(range(0, cs.count, k))
    sub = fg.ClusterSet.from_lists([cs.vertices[cs.off[c]:cs.off[c + 1]] for c in pick],
                                   [cs.borders[cs.boff[c]:cs.boff[c + 1]] for c in pick])
    mw = _mean_weight(g)
    best, arg = float("inf"), None
    for dm, ch, bt in itertools.product(deltas, chunks, threads):
        choice = {"delta": max(1, int(round(dm * mw))), "chunk_max": ch, "frontier_threads": bt}
        _apply(choice)
        t = _time(lambda st: fg.cluster_eval_batch(g, sub, precision, fg.BATCHED, stats=st))
        if t < best:
            best, arg = t, choice
    return _apply(arg)

"""Python binding of the GB300 Brandes engine (ctypes over ``libfbcgpu.so``).

The classes mirror the reference's hot-path interfaces, with the same names, argument
meaning and error behaviour, so tests and callers read like the reference's own code:

  ExactBrandesBC.computeBC(graph)                         IBrandesBC.h:24, ExactBrandesBC.h:45-95
  DijkstraSSBrandesBC.singleSourceBrandes(source, graph)  ISSBrandesBC.h:26-28, DijkstraSSBrandesBC.h:45-81
  DijkstraClusterEvaluator.evaluateCluster(clusterBC, globalVI, cluster)
                                                          IClusterEvaluator.h:33-36,
                                                          DijkstraClusterEvaluator.h:50-180
Batched forms (one call per phase instead of one per source) are exposed as functions.

Errors: every C status other than FBC_OK raises ``FbcError`` (a RuntimeError) carrying the
library's message; invalid input raises before the device is touched, as the reference's
``std::invalid_argument`` does.  There is no CPU fallback: if the shared library is missing
this module fails at import time.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libfbcgpu.so")

FBC_OK = 0
FBC_ERR_INVALID_ARG = 1
FBC_ERR_CUDA = 2
FBC_ERR_OOM = 3
FBC_ERR_ITER_LIMIT = 4
FBC_ERR_RANGE = 5
FBC_ERR_SIGMA_OVERFLOW = 6
FBC_ERR_NOT_INIT = 7
FBC_ERR_QUEUE = 8
FBC_ERR_HASH = 9

FP64 = 0
FP32C = 1
PLAIN = 0
BATCHED = 1


class FbcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"fbc error {code}: {msg}")
        self.code = code


class Stats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("wall_ms", C.c_double), ("h2d_bytes", C.c_int64),
                ("d2h_bytes", C.c_int64), ("units", C.c_int64), ("relaxations", C.c_double),
                ("launches", C.c_int32), ("slots", C.c_int32), ("warp_ms", C.c_double),
                ("block_ms", C.c_double), ("warp_bytes", C.c_double), ("block_bytes", C.c_double),
                ("warp_units", C.c_int64), ("block_units", C.c_int64), ("group", C.c_int32),
                ("retries", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
    lib = C.CDLL(LIB_PATH)
    P = C.POINTER
    i32, i64, dbl, vp = C.c_int32, C.c_int64, C.c_double, C.c_void_p
    sig = {
        "fbc_gpu_init": ([C.c_int], C.c_int),
        "fbc_gpu_shutdown": ([], C.c_int),
        "fbc_last_error_string": ([], C.c_char_p),
        "fbc_set_option": ([C.c_char_p, i64], C.c_int),
        "fbc_get_option": ([C.c_char_p, P(i64)], C.c_int),
        "fbc_graph_upload": ([i32, vp, vp, vp, P(vp)], C.c_int),
        "fbc_graph_from_edges": ([i64, vp, vp, vp, P(vp)], C.c_int),
        "fbc_graph_from_text": ([C.c_char_p, i64, P(vp), P(Stats)], C.c_int),
        "fbc_graph_info": ([vp, P(i32), P(i64)], C.c_int),
        "fbc_graph_download": ([vp, vp, vp, vp], C.c_int),
        "fbc_graph_free": ([vp], C.c_int),
        "fbc_exact_bc": ([vp, C.c_int, C.c_int, vp, P(Stats)], C.c_int),
        "fbc_single_source": ([vp, i32, C.c_int, vp, P(Stats)], C.c_int),
        "fbc_sssp_dependency_batch": ([vp, i64, vp, vp, C.c_int, C.c_int, vp, P(Stats)], C.c_int),
        "fbc_cluster_border_count": ([vp, i32, vp, vp, vp, P(i64), P(i64)], C.c_int),
        "fbc_cluster_borders": ([vp, i32, vp, vp, vp, vp], C.c_int),
        "fbc_cluster_eval_batch": ([vp, i32, vp, vp, vp, vp, C.c_int, C.c_int, vp, vp, vp,
                                    P(Stats)], C.c_int),
        "fbc_multi_exact_bc": ([i32, vp, C.c_int, C.c_int, vp, P(Stats)], C.c_int),
        "fbc_sssp_debug": ([vp, i32, vp, vp, vp, vp], C.c_int),
        "fbc_cluster_classes": ([vp, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp], C.c_int),
        "fbc_cluster_plan_create": ([vp, i32, vp, vp, vp, vp, C.c_int, P(vp)], C.c_int),
        "fbc_plan_run": ([vp, P(Stats)], C.c_int),
        "fbc_plan_results": ([vp, P(vp), P(vp), P(vp), P(i64), P(i32)], C.c_int),
        "fbc_plan_free": ([vp], C.c_int),
        "fbc_kmeans": ([i32, vp, vp, vp, vp, vp, vp, vp, dbl, i32, vp, vp, P(Stats)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    lib.signatures = sig
    return lib


lib = _load()


def _ck(rc: int) -> None:
    if rc != FBC_OK:
        msg = lib.fbc_last_error_string()
        raise FbcError(rc, msg.decode() if msg else "")


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


_initialised = False


def init(device: int = 0) -> None:
    """Select the CUDA device and create the library stream (idempotent)."""
    global _initialised
    if not _initialised:
        _ck(lib.fbc_gpu_init(device))
        _initialised = True


def shutdown() -> None:
    global _initialised
    _ck(lib.fbc_gpu_shutdown())
    _initialised = False


def set_option(key: str, value: int) -> None:
    _ck(lib.fbc_set_option(key.encode(), int(value)))


def get_option(key: str) -> int:
    v = C.c_int64()
    _ck(lib.fbc_get_option(key.encode(), C.byref(v)))
    return v.value


class Graph:
    """A device-resident directed weighted graph (the GPU form of DirectedWeightedGraph)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        n, m = C.c_int32(), C.c_int64()
        _ck(lib.fbc_graph_info(self._h, C.byref(n), C.byref(m)))
        self.n, self.m = n.value, m.value

    @classmethod
    def from_csr(cls, row_ptr, col, w) -> "Graph":
        init()
        rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
        cl = np.ascontiguousarray(col, dtype=np.int32)
        ww = np.ascontiguousarray(w, dtype=np.float64)
        h = C.c_void_p()
        _ck(lib.fbc_graph_upload(rp.size - 1, _ptr(rp), _ptr(cl), _ptr(ww), C.byref(h)))
        return cls(h)

    @classmethod
    def from_edges(cls, src, dst, w) -> "Graph":
        """Edge-list rules of the reference parser: weights of repeated pairs summed,
        n = 1 + max source id, weight <= 0 rejected."""
        init()
        s = np.ascontiguousarray(src, dtype=np.int32)
        d = np.ascontiguousarray(dst, dtype=np.int32)
        ww = np.ascontiguousarray(w, dtype=np.float64)
        h = C.c_void_p()
        _ck(lib.fbc_graph_from_edges(s.size, _ptr(s), _ptr(d), _ptr(ww), C.byref(h)))
        return cls(h)

    @classmethod
    def from_edgelist(cls, el) -> "Graph":
        rp, col, w = el.csr()
        return cls.from_csr(rp, col, w.astype(np.float64))

    @classmethod
    def from_text(cls, data: bytes, stats: Stats | None = None) -> "Graph":
        """Edge-list text ("src dst weight" triples, the file format fbc reads), tokenised and
        parsed on the device with the reference parser's rules (fbc_graph_from_text)."""
        init()
        data = bytes(data)
        h = C.c_void_p()
        _ck(lib.fbc_graph_from_text(data, len(data), C.byref(h), _stats(stats)))
        return cls(h)

    @classmethod
    def from_file(cls, path: str) -> "Graph":
        with open(path, "rb") as f:
            return cls.from_text(f.read())

    def csr(self):
        rp = np.zeros(self.n + 1, np.int64)
        col = np.zeros(max(self.m, 1), np.int32)
        w = np.zeros(max(self.m, 1), np.float64)
        _ck(lib.fbc_graph_download(self._h, _ptr(rp), _ptr(col), _ptr(w)))
        return rp, col[: self.m], w[: self.m]

    def vertices(self) -> np.ndarray:
        return np.arange(self.n, dtype=np.int32)

    def edges(self) -> int:
        return self.m

    def free(self) -> None:
        if self._h:
            lib.fbc_graph_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _stats(st: Stats | None):
    return C.byref(st) if st is not None else None


def exact_bc(g: Graph, precision: int = FP64, sched: int = PLAIN, stats: Stats | None = None):
    out = np.zeros(max(g.n, 1), np.float64)
    _ck(lib.fbc_exact_bc(g._h, precision, sched, _ptr(out), _stats(stats)))
    return out[: g.n]


def single_source(g: Graph, source: int, precision: int = FP64, stats: Stats | None = None):
    out = np.zeros(max(g.n, 1), np.float64)
    _ck(lib.fbc_single_source(g._h, int(source), precision, _ptr(out), _stats(stats)))
    return out[: g.n]


def dependency_batch(g: Graph, sources, cards=None, precision: int = FP64, sched: int = PLAIN,
                     out: np.ndarray | None = None, stats: Stats | None = None):
    """out[v] += sum_p cards[p] * dep_p[v] (the pivot loop, ClusteredBrandesBC.h:141-155)."""
    s = np.ascontiguousarray(sources, dtype=np.int32)
    c = None if cards is None else np.ascontiguousarray(cards, dtype=np.float64)
    if out is None:
        out = np.zeros(max(g.n, 1), np.float64)
    _ck(lib.fbc_sssp_dependency_batch(g._h, s.size, _ptr(s), _ptr(c), precision, sched, _ptr(out),
                                      _stats(stats)))
    return out[: g.n]


@dataclass
class ClusterSet:
    """Clusters as flat arrays: cluster c = vertices[off[c]:off[c+1]] (the community order),
    borders bl[boff[c]:boff[c+1]] ascending (SubGraph::borders)."""
    off: np.ndarray
    vertices: np.ndarray
    boff: np.ndarray | None = None
    borders: np.ndarray | None = None

    @classmethod
    def from_lists(cls, clusters, borders=None) -> "ClusterSet":
        off = np.zeros(len(clusters) + 1, np.int64)
        off[1:] = np.cumsum([len(c) for c in clusters])
        verts = np.concatenate([np.asarray(c, np.int32) for c in clusters]) if clusters else \
            np.zeros(0, np.int32)
        bo = bl = None
        if borders is not None:
            bo = np.zeros(len(borders) + 1, np.int64)
            bo[1:] = np.cumsum([len(b) for b in borders])
            bl = np.concatenate([np.asarray(b, np.int32) for b in borders]) if borders else \
                np.zeros(0, np.int32)
        return cls(off, verts.astype(np.int32), bo, bl)

    @property
    def count(self) -> int:
        return self.off.size - 1

    def with_borders(self, g: Graph) -> "ClusterSet":
        if self.boff is not None:
            return self
        bo = np.zeros(self.count + 1, np.int64)
        bl = np.zeros(max(g.n, 1), np.int32)
        _ck(lib.fbc_cluster_borders(g._h, self.count, _ptr(self.off), _ptr(self.vertices),
                                    _ptr(bo), _ptr(bl)))
        return ClusterSet(self.off, self.vertices, bo, bl[: bo[-1]].copy())


@dataclass
class ClusterEval:
    intra_bc: np.ndarray
    border_dist: np.ndarray
    border_sigma: np.ndarray
    clusters: ClusterSet
    entry_off: np.ndarray = field(default=None)

    def vertex_info(self, c: int, i: int):
        """(lengths, counts) of the i-th vertex of cluster c over its borders."""
        nb = int(self.clusters.boff[c + 1] - self.clusters.boff[c])
        e = int(self.entry_off[c]) + i * nb
        return self.border_dist[e:e + nb], self.border_sigma[e:e + nb]


def cluster_eval_batch(g: Graph, cs: ClusterSet, precision: int = FP64, sched: int = PLAIN,
                       intra_bc: np.ndarray | None = None, stats: Stats | None = None,
                       out: "ClusterEval | None" = None) -> ClusterEval:
    """Evaluate every cluster (DijkstraClusterEvaluator::evaluateCluster for all of them).
    `out`: a ClusterEval of an earlier call on the same clusters whose arrays are reused (a
    repeated sweep then writes into memory that is already mapped); intra_bc is added to."""
    cs = cs.with_borders(g)
    nb = np.diff(cs.boff)
    sizes = np.diff(cs.off)
    entry_off = np.zeros(cs.count + 1, np.int64)
    entry_off[1:] = np.cumsum(nb * sizes)
    ent = int(entry_off[-1])
    if out is not None and out.border_dist.size == ent and out.border_sigma.size == ent and ent > 0:
        bd, bs = out.border_dist, out.border_sigma
        if intra_bc is None:
            intra_bc = out.intra_bc
            intra_bc[:] = 0.0
    else:
        bd = np.zeros(max(ent, 1), np.float64)
        bs = np.zeros(max(ent, 1), np.uint64)
    if intra_bc is None:
        intra_bc = np.zeros(max(g.n, 1), np.float64)
    _ck(lib.fbc_cluster_eval_batch(g._h, cs.count, _ptr(cs.off), _ptr(cs.vertices), _ptr(cs.boff),
                                   _ptr(cs.borders if cs.borders.size else np.zeros(1, np.int32)),
                                   precision, sched, _ptr(intra_bc), _ptr(bd), _ptr(bs),
                                   _stats(stats)))
    return ClusterEval(intra_bc[: g.n], bd[:ent], bs[:ent], cs, entry_off)


class ClusterPlan:
    """A prepared cluster sweep (fbc_cluster_plan_create): the cluster subgraphs are uploaded
    once and each run() replays captured CUDA graphs of the sweep's kernels (the shared-memory
    kernel and/or the frontier kernel, by community size)."""

    def __init__(self, g: Graph, cs: ClusterSet, precision: int = FP64):
        self.g = g
        self.cs = cs.with_borders(g)
        nb = np.diff(self.cs.boff)
        self.entry_off = np.zeros(self.cs.count + 1, np.int64)
        self.entry_off[1:] = np.cumsum(nb * np.diff(self.cs.off))
        h = C.c_void_p()
        bl = self.cs.borders if self.cs.borders.size else np.zeros(1, np.int32)
        _ck(lib.fbc_cluster_plan_create(g._h, self.cs.count, _ptr(self.cs.off), _ptr(self.cs.vertices),
                                        _ptr(self.cs.boff), _ptr(bl), precision, C.byref(h)))
        self._h = h

    @property
    def captured(self) -> bool:
        cap = C.c_int32()
        _ck(lib.fbc_plan_results(self._h, None, None, None, None, C.byref(cap)))
        return bool(cap.value)

    def run(self, stats: Stats | None = None, copy: bool = True) -> ClusterEval:
        """Replay the sweep.  With copy=False the returned arrays are views of the plan's pinned
        buffers, overwritten by the next run."""
        _ck(lib.fbc_plan_run(self._h, _stats(stats)))
        bcp, bdp, bsp = C.c_void_p(), C.c_void_p(), C.c_void_p()
        ent = C.c_int64()
        _ck(lib.fbc_plan_results(self._h, C.byref(bcp), C.byref(bdp), C.byref(bsp), C.byref(ent), None))
        n, e = self.g.n, int(ent.value)
        bc = np.ctypeslib.as_array(C.cast(bcp, C.POINTER(C.c_double)), (max(n, 1),))[:n]
        bd = np.ctypeslib.as_array(C.cast(bdp, C.POINTER(C.c_double)), (max(e, 1),))[:e]
        bs = np.ctypeslib.as_array(C.cast(bsp, C.POINTER(C.c_uint64)), (max(e, 1),))[:e]
        if copy:
            bc, bd, bs = bc.copy(), bd.copy(), bs.copy()
        return ClusterEval(bc, bd, bs, self.cs, self.entry_off)

    def free(self) -> None:
        if getattr(self, "_h", None):
            lib.fbc_plan_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def cluster_classes(g: Graph, cs: ClusterSet, bc, ev: ClusterEval):
    """VertexInfoPivotSelector::selectPivots for every cluster (exact topological classes):
    per cluster, (pivots, cardinalities) in class order.  `bc` is the BC the selection compares
    (the intra-cluster BC), `ev` the border vectors of a cluster_eval_batch on the same clusters."""
    cs = cs.with_borders(g)
    bcv = np.ascontiguousarray(bc, np.float64)
    coff = np.zeros(cs.count + 1, np.int64)
    piv = np.zeros(max(int(cs.off[-1]), 1), np.int32)
    crd = np.zeros(max(int(cs.off[-1]), 1), np.int32)
    bl = cs.borders if cs.borders.size else np.zeros(1, np.int32)
    bd = ev.border_dist if ev.border_dist.size else np.zeros(1)
    bs = ev.border_sigma if ev.border_sigma.size else np.zeros(1, np.uint64)
    _ck(lib.fbc_cluster_classes(g._h, cs.count, _ptr(cs.off), _ptr(cs.vertices), _ptr(cs.boff), _ptr(bl),
                                _ptr(bcv), _ptr(np.ascontiguousarray(bd)), _ptr(np.ascontiguousarray(bs)),
                                _ptr(coff), _ptr(piv), _ptr(crd)))
    return [(piv[coff[c]:coff[c + 1]].copy(), crd[coff[c]:coff[c + 1]].copy()) for c in range(cs.count)]


def kmeans(sets, kfrac: float = 0.5, max_iter: int = 100, min_variance: float = 0.0,
           stats: Stats | None = None):
    """PlusPlusKMeans::computeCentroids on the device for several point sets at once (fbc_kmeans).
    `sets`: (lengths np x nb, counts np x nb, weights np) per set, the normalized border vectors of
    the exact classes' pivots and the class sizes; k = max(int(np * kfrac), 1) as
    KMeansPivotSelector chooses it.  Returns per set (centroid point indices, weights), duplicates
    kept."""
    nsets = len(sets)
    set_off = np.zeros(nsets + 1, np.int64)
    nb = np.zeros(max(nsets, 1), np.int32)
    vec_off = np.zeros(max(nsets, 1), np.int64)
    ks = np.zeros(max(nsets, 1), np.int32)
    Ls, Cs, Ws = [], [], []
    vo = 0
    for s, (L, Cn, w) in enumerate(sets):
        L = np.ascontiguousarray(L, np.float64)
        npv = L.shape[0]
        set_off[s + 1] = set_off[s] + npv
        nb[s] = L.shape[1] if L.ndim == 2 else 0
        vec_off[s] = vo
        vo += L.size
        ks[s] = max(int(npv * kfrac), 1)
        Ls.append(L.ravel())
        Cs.append(np.ascontiguousarray(Cn, np.int32).ravel())
        Ws.append(np.ascontiguousarray(w, np.int32))
    Lf = np.concatenate(Ls) if vo else np.zeros(1)
    Cf = np.concatenate(Cs) if vo else np.zeros(1, np.int32)
    Wf = np.concatenate(Ws) if nsets else np.zeros(1, np.int32)
    kout = np.zeros(max(int(ks[:nsets].sum()), 1), np.int32)
    wout = np.zeros_like(kout)
    _ck(lib.fbc_kmeans(nsets, _ptr(set_off), _ptr(nb), _ptr(vec_off), _ptr(Lf), _ptr(Cf), _ptr(Wf), _ptr(ks),
                       float(min_variance), int(max_iter), _ptr(kout), _ptr(wout), _stats(stats)))
    out, o = [], 0
    for s in range(nsets):
        out.append((kout[o:o + ks[s]].copy(), wout[o:o + ks[s]].copy()))
        o += ks[s]
    return out


def kmeans_pivot_sets(class_pivots, sets, kfrac: float = 0.5, max_iter: int = 100):
    """KMeansPivotSelector::selectPivots after the exact classes (KMeansPivotSelector.h:92-130):
    the device k-means, then duplicate pivots removed keeping the first; `class_pivots[s]` maps a
    set's point index to its vertex.  Returns per set (pivots, weights)."""
    res = []
    for cp, (idx, w) in zip(class_pivots, kmeans(sets, kfrac, max_iter)):
        seen, pv, pw = set(), [], []
        for i, x in zip(idx.tolist(), w.tolist()):
            if i in seen:
                continue
            seen.add(i)
            pv.append(int(cp[i]))
            pw.append(x)
        res.append((np.array(pv, np.int32), np.array(pw, np.int32)))
    return res


def multi_exact_bc(graphs: list[Graph], precision: int = FP64, sched: int = BATCHED,
                   stats: Stats | None = None) -> list[np.ndarray]:
    outs = [np.zeros(max(gr.n, 1), np.float64) for gr in graphs]
    hs = (C.c_void_p * len(graphs))(*[gr._h for gr in graphs])
    ps = (C.c_void_p * len(graphs))(*[o.ctypes.data for o in outs])
    _ck(lib.fbc_multi_exact_bc(len(graphs), C.cast(hs, C.c_void_p), precision, sched,
                               C.cast(ps, C.c_void_p), _stats(stats)))
    return [o[: gr.n] for o, gr in zip(outs, graphs)]


def sssp_debug(g: Graph, source: int):
    """(dist int32 with -1 = unreached, sigma uint64, delta float64, npred int32)."""
    dist = np.zeros(max(g.n, 1), np.int32)
    sig = np.zeros(max(g.n, 1), np.uint64)
    dlt = np.zeros(max(g.n, 1), np.float64)
    npred = np.zeros(max(g.n, 1), np.int32)
    _ck(lib.fbc_sssp_debug(g._h, int(source), _ptr(dist), _ptr(sig), _ptr(dlt), _ptr(npred)))
    return dist[: g.n], sig[: g.n], dlt[: g.n], npred[: g.n]


def clustered_bc(g: Graph, cs: ClusterSet, pivots: list, cards: list, precision: int = FP64,
                 sched: int = PLAIN, ev: ClusterEval | None = None, stats: list | None = None):
    """The GPU phases of ClusteredBrandeBC::computeBC (ClusteredBrandesBC.h:63-169) for a given
    partition and pivot set (both produced by the reference's host code): intra-cluster BC,
    then BC += sum_p dep_p * card_p and BC[v in C] -= intraBC[v] * sum_{p in C} card_p."""
    st1, st2 = Stats(), Stats()
    if ev is None:
        ev = cluster_eval_batch(g, cs, precision, sched, stats=st1)
    bc = ev.intra_bc.copy()
    allp = np.concatenate([np.asarray(p, np.int32) for p in pivots]) if pivots else np.zeros(0, np.int32)
    allc = np.concatenate([np.asarray(c, np.float64) for c in cards]) if cards else np.zeros(0)
    dependency_batch(g, allp, allc, precision, sched, out=bc, stats=st2)
    # BC[v] -= intraBC[v] * (summed cardinalities of v's cluster's pivots), all clusters at once
    tot = np.array([float(np.sum(np.asarray(cards[c], np.float64))) if len(cards[c]) else 0.0
                    for c in range(cs.count)])
    mult = np.zeros(g.n)
    mult[cs.vertices] = np.repeat(tot, np.diff(cs.off))
    bc -= ev.intra_bc * mult
    if stats is not None:
        stats.extend([st1, st2])
    return bc


def write_bc(path: str, bc) -> None:
    """The fbc CLI's result file (main.cpp:123-130, 282-294): one value per line as an ostream
    prints a double (six significant digits, the %g form), entries that are not >= 0 written
    as 0; an existing file is refused (FileExistsError), as the CLI refuses it."""
    with open(path, "x") as f:
        f.write("".join(("%g\n" % x) if x >= 0 else "0\n" for x in np.asarray(bc, np.float64).tolist()))

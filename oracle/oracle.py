"""ctypes front end of the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE ONLY.

Restates the reference's Brandes hot path (see brandes_oracle.h for the file:line map).
Imported only by the test suite, the smoke check and the benchmark's CPU-baseline leg,
always as the checker or the CPU baseline, never as a compute path of the GPU library.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} missing: run make -C oracle")
        L = C.CDLL(LIB_PATH)
        vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
        L.orc_exact_bc.argtypes = [i32, vp, vp, vp, vp, C.c_int]
        L.orc_exact_bc_sources.argtypes = [i32, vp, vp, vp, i64, vp, vp, C.c_int]
        L.orc_single_source.argtypes = [i32, vp, vp, vp, i32, vp]
        L.orc_sssp_dump.argtypes = [i32, vp, vp, vp, i32, vp, vp, vp, vp, vp, vp]
        L.orc_sssp_dump.restype = i64
        L.orc_cluster_eval.argtypes = [i32, vp, vp, vp, i32, vp, i32, vp, vp, vp, vp, C.c_int]
        L.orc_pivot_batch.argtypes = [i32, vp, vp, vp, i64, vp, vp, vp, C.c_int]
        L.orc_kmeans_pivots.argtypes = [i32, i32, vp, vp, vp, C.c_double, i32, vp, vp]
        L.orc_kmeans_pivots.restype = i32
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class CSR:
    """Host CSR with double weights (W=double)."""

    def __init__(self, row_ptr, col, w):
        self.rp = np.ascontiguousarray(row_ptr, np.int64)
        self.col = np.ascontiguousarray(col, np.int32)
        self.w = np.ascontiguousarray(w, np.float64)
        self.n = self.rp.size - 1
        self.m = int(self.rp[-1])

    @classmethod
    def from_edgelist(cls, el):
        rp, col, w = el.csr()
        return cls(rp, col, w.astype(np.float64))

    def args(self):
        return (self.n, _p(self.rp), _p(self.col), _p(self.w))


def exact_bc(g: CSR, threads: int = 1) -> np.ndarray:
    out = np.zeros(max(g.n, 1))
    assert lib().orc_exact_bc(*g.args(), _p(out), threads) == 0
    return out[: g.n]


def exact_bc_sources(g: CSR, sources, threads: int = 1) -> np.ndarray:
    s = np.ascontiguousarray(sources, np.int32)
    out = np.zeros(max(g.n, 1))
    assert lib().orc_exact_bc_sources(*g.args(), s.size, _p(s), _p(out), threads) == 0
    return out[: g.n]


def single_source(g: CSR, src: int) -> np.ndarray:
    out = np.zeros(max(g.n, 1))
    assert lib().orc_single_source(*g.args(), int(src), _p(out)) == 0
    return out[: g.n]


def sssp_dump(g: CSR, src: int):
    """dist (inf when unreached), sigma, delta, settle order, predecessor lists."""
    n = g.n
    dist, sig, dlt = np.zeros(n), np.zeros(n), np.zeros(n)
    order = np.zeros(n, np.int32)
    poff = np.zeros(n + 1, np.int64)
    cnt = lib().orc_sssp_dump(*g.args(), int(src), None, None, None, None, _p(poff), None)
    pred = np.zeros(max(int(poff[-1]), 1), np.int32)
    cnt = lib().orc_sssp_dump(*g.args(), int(src), _p(dist), _p(sig), _p(dlt), _p(order), _p(poff),
                              _p(pred))
    assert cnt >= 0
    dist[dist == np.finfo(np.float64).max] = np.inf
    preds = [pred[poff[v]:poff[v + 1]].copy() for v in range(n)]
    return dist, sig, dlt, order[:cnt], preds


def cluster_eval(g: CSR, verts, borders, bc_accum=None, threads: int = 1):
    v = np.ascontiguousarray(verts, np.int32)
    b = np.ascontiguousarray(borders, np.int32)
    if bc_accum is None:
        bc_accum = np.zeros(max(g.n, 1))
    bd = np.zeros(max(v.size * b.size, 1))
    bs = np.zeros(max(v.size * b.size, 1))
    assert lib().orc_cluster_eval(*g.args(), v.size, _p(v), b.size, _p(b), _p(bc_accum), _p(bd),
                                  _p(bs), threads) == 0
    return bc_accum, bd[: v.size * b.size].reshape(v.size, b.size), \
        bs[: v.size * b.size].reshape(v.size, b.size)


def pivot_batch(g: CSR, pivots, cards, bc_accum=None, threads: int = 1):
    p = np.ascontiguousarray(pivots, np.int32)
    c = np.ascontiguousarray(cards, np.float64)
    if bc_accum is None:
        bc_accum = np.zeros(max(g.n, 1))
    assert lib().orc_pivot_batch(*g.args(), p.size, _p(p), _p(c), _p(bc_accum), threads) == 0
    return bc_accum


def kmeans_pivots(lengths, counts, weights, kfrac: float = 0.5, max_iter: int = 100):
    """KMeansPivotSelector's k-means step on one cluster's exact classes: lengths / counts are the
    class pivots' normalized border vectors (np x b), weights the class sizes.  Returns (indices
    into the class list, weights) of the distinct chosen pivots."""
    L = np.ascontiguousarray(lengths, np.float64)
    Cn = np.ascontiguousarray(counts, np.int32)
    w = np.ascontiguousarray(weights, np.int32)
    npv = L.shape[0]
    b = L.shape[1] if L.ndim == 2 else 0
    k = max(int(npv * kfrac), 1)
    idx = np.zeros(k, np.int32)
    ow = np.zeros(k, np.int32)
    cnt = lib().orc_kmeans_pivots(npv, b, _p(L), _p(Cn), _p(w), kfrac, max_iter, _p(idx), _p(ow))
    return idx[:cnt], ow[:cnt]

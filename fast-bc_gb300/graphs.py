"""Seeded synthetic graph generators for the betweenness workloads.

Every generator is a pure function of its arguments: the random stream is a
counter-based splitmix64 hash evaluated with numpy uint64 arithmetic, so the same
call yields the same edge list on x86 and on Arm, and across numpy versions
(no numpy Generator is involved).

Edge-list semantics follow the reference parser (DirectedWeightedGraph.h:67-96):
one ``src dst w`` line per directed edge, vertex count = 1 + max source id.
Each generator writes every directed pair at most once (the reference would sum
the weights of a repeated pair, DirectedWeightedGraph.h:154-165) and makes sure
the highest vertex id has an out-edge, so the vertex count is the intended one.

Workloads (sizes as named by the benchmark configurations):
  * ``road_grid(32, 32, drop=0, highway=0)``            -> 1,024 vertices, 3,968 edges
  * ``road_grid(256, 256)``                             -> clustered 256x256 road grid
  * ``road_grid(512, 512)``                             -> 262,144-vertex precision grid
  * ``road_grid(2048, 2048, highway=0.001, radius=128)`` -> 4,194,304-vertex road grid
  * ``rgg_batch(48)``                                   -> 48 random geometric 3-NN graphs
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

_U = np.uint64
_GOLD = _U(0x9E3779B97F4A7C15)


def _mix(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser (Steele, Lea, Flood 2014), elementwise on uint64."""
    with np.errstate(over="ignore"):
        x = x + _GOLD
        x = (x ^ (x >> _U(30))) * _U(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> _U(27))) * _U(0x94D049BB133111EB)
        return x ^ (x >> _U(31))


def rand_u64(seed: int, stream: int, idx) -> np.ndarray:
    """Counter-based 64-bit random words: one per element of ``idx``."""
    idx = np.asarray(idx, dtype=np.uint64)
    key = _mix(np.array([(seed * 0x100000001B3 + stream * 0x5851F42D4C957F2D) & 0xFFFFFFFFFFFFFFFF],
                        dtype=np.uint64))[0]
    with np.errstate(over="ignore"):
        return _mix(idx * _U(0xD1B54A32D192ED03) ^ key)


def rand_int(seed: int, stream: int, idx, lo: int, hi: int) -> np.ndarray:
    """Integers uniform in [lo, hi] (inclusive)."""
    span = _U(hi - lo + 1)
    return (rand_u64(seed, stream, idx) % span).astype(np.int64) + lo


def rand_unit(seed: int, stream: int, idx) -> np.ndarray:
    """Doubles uniform in [0, 1): the top 53 bits of the random word."""
    return (rand_u64(seed, stream, idx) >> _U(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclass
class EdgeList:
    """A directed weighted edge list, sorted by (src, dst), pairs unique."""
    n: int
    src: np.ndarray  # int32
    dst: np.ndarray  # int32
    w: np.ndarray    # int32 (positive)

    @property
    def m(self) -> int:
        return int(self.src.shape[0])

    def write(self, path: str) -> None:
        """Write the ``src dst w`` text form read by the reference ``fbc``."""
        with open(path, "wb") as f:
            f.write(self.text())

    def text(self) -> bytes:
        """The ``src dst w`` lines (decimal, one space, "\n") as bytes, formatted with array
        operations: every number is written into a fixed-width field of digit bytes (as wide as
        its column's largest value), and the unused leading positions are dropped."""
        cols = [self.src, self.dst, self.w]
        widths = [len(str(int(x.max()))) + 1 if x.size else 2 for x in cols]
        m, tot = self.m, sum(widths)
        buf = np.empty((m, tot), np.uint8)
        keep = np.empty((m, tot), bool)
        base = 0
        for c, x in enumerate(cols):
            y = x.astype(np.int32)
            assert y.size == 0 or y.min() >= 0
            wd = widths[c]
            started = np.ones(m, bool)  # the lowest digit is always written
            for k in range(wd - 1):  # digit k from the right
                pos = base + wd - 2 - k
                buf[:, pos] = 48 + (y % 10).astype(np.uint8)
                keep[:, pos] = started
                y = y // 10
                started = y > 0
            buf[:, base + wd - 1] = 32 if c < 2 else 10
            keep[:, base + wd - 1] = True
            base += wd
        return buf[keep].tobytes()

    def csr(self):
        """CSR arrays (row_ptr int64[n+1], col int32[m], w int32[m]); neighbours ascending."""
        order = np.lexsort((self.dst, self.src))
        src, dst, w = self.src[order], self.dst[order], self.w[order]
        counts = np.bincount(src, minlength=self.n)
        row_ptr = np.zeros(self.n + 1, dtype=np.int64)
        np.cumsum(counts, out=row_ptr[1:])
        return row_ptr, dst.astype(np.int32), w.astype(np.int32)


def _finish(n: int, s: np.ndarray, d: np.ndarray, w: np.ndarray) -> EdgeList:
    order = np.lexsort((d, s))
    s, d, w = s[order], d[order], w[order]
    if s.size:
        key = s.astype(np.int64) * n + d
        assert np.all(np.diff(key) > 0), "generator produced a repeated directed pair"
        assert int(s.max()) == n - 1, "highest vertex id must have an out-edge"
    return EdgeList(n, s.astype(np.int32), d.astype(np.int32), w.astype(np.int32))


def road_grid(rows: int, cols: int, *, drop: float = 0.05, highway: float = 0.002,
              radius: int = 32, wmax: int = 100, hw_wmax: int = 20, seed: int = 42) -> EdgeList:
    """Road-like 4-neighbour grid, ids row-major.

    Each undirected neighbour pair is dropped with probability ``drop``; a kept pair
    becomes two directed edges with independent weights uniform in [1, wmax].  A
    fraction ``highway`` of the vertices gets one extra bidirectional edge to a vertex
    drawn uniformly within Manhattan distance ``radius`` (weights uniform in
    [1, hw_wmax]); a highway that repeats an existing pair is skipped.
    """
    n = rows * cols
    r = np.arange(rows, dtype=np.int64)
    c = np.arange(cols, dtype=np.int64)
    # horizontal pairs (r,c)-(r,c+1) and vertical pairs (r,c)-(r+1,c)
    ha = (r[:, None] * cols + c[None, :-1]).ravel()
    va = (r[:-1, None] * cols + c[None, :]).ravel()
    a = np.concatenate([ha, va])
    b = np.concatenate([ha + 1, va + cols])
    pid = np.arange(a.size, dtype=np.int64)
    keep = rand_unit(seed, 1, pid) >= drop
    # the last vertex keeps its horizontal pair so that n = rows*cols (n = 1 + max src)
    if cols > 1:
        keep[(rows - 1) * (cols - 1) + (cols - 2)] = True
    elif rows > 1:
        keep[-1] = True
    a, b, pid = a[keep], b[keep], pid[keep]
    w_ab = rand_int(seed, 2, 2 * pid, 1, wmax)
    w_ba = rand_int(seed, 2, 2 * pid + 1, 1, wmax)
    src = [a, b]
    dst = [b, a]
    wts = [w_ab, w_ba]

    if highway > 0:
        vid = np.arange(n, dtype=np.int64)
        chosen = vid[rand_unit(seed, 5, vid) < highway]
        tgt = np.full(chosen.size, -1, dtype=np.int64)
        for attempt in range(64):
            todo = tgt < 0
            if not todo.any():
                break
            k = chosen[todo] * 64 + attempt
            dr = rand_int(seed, 6, k, -radius, radius)
            dc = rand_int(seed, 7, k, -radius, radius)
            rr = chosen[todo] // cols + dr
            cc = chosen[todo] % cols + dc
            ok = ((np.abs(dr) + np.abs(dc)) <= radius) & ((dr != 0) | (dc != 0)) \
                & (rr >= 0) & (rr < rows) & (cc >= 0) & (cc < cols)
            cand = np.where(ok, rr * cols + cc, -1)
            sub = tgt[todo]
            sub[ok] = cand[ok]
            tgt[todo] = sub
        good = tgt >= 0
        ha_, hb_ = chosen[good], tgt[good]
        lo, hi = np.minimum(ha_, hb_), np.maximum(ha_, hb_)
        existing = np.minimum(a, b) * n + np.maximum(a, b)
        key = lo * n + hi
        _, first = np.unique(key, return_index=True)
        uniq = np.zeros(key.size, dtype=bool)
        uniq[first] = True
        fresh = uniq & ~np.isin(key, existing)
        ha_, hb_ = ha_[fresh], hb_[fresh]
        hid = np.flatnonzero(good)[fresh].astype(np.int64)
        hw1 = rand_int(seed, 8, 2 * hid, 1, hw_wmax)
        hw2 = rand_int(seed, 8, 2 * hid + 1, 1, hw_wmax)
        src += [ha_, hb_]
        dst += [hb_, ha_]
        wts += [hw1, hw2]
    return _finish(n, np.concatenate(src), np.concatenate(dst), np.concatenate(wts))


def rgg_knn(n: int, *, k: int = 3, seed: int = 7, gid: int = 0) -> EdgeList:
    """Random geometric graph: points uniform in the unit square, each point joined to
    its ``k`` nearest neighbours by edges in both directions, weight = ceil(1000 * d).
    Mutual neighbours give one pair, not two (no summed weights).
    The highest id gets an out-edge by construction (every point has k neighbours)."""
    from scipy.spatial import cKDTree

    idx = np.arange(n, dtype=np.int64)
    x = rand_unit(seed, 100 + 2 * gid, idx)
    y = rand_unit(seed, 101 + 2 * gid, idx)
    pts = np.stack([x, y], axis=1)
    _, nb = cKDTree(pts).query(pts, k=k + 1)
    nb = nb[:, 1:].astype(np.int64)
    a = np.repeat(idx, k)
    b = nb.ravel()
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    key = np.unique(lo * n + hi)
    lo, hi = key // n, key % n
    dx = x[lo] - x[hi]
    dy = y[lo] - y[hi]
    d = np.sqrt(dx * dx + dy * dy)
    w = np.ceil(1000.0 * d).astype(np.int64)
    w = np.maximum(w, 1)
    return _finish(n, np.concatenate([lo, hi]), np.concatenate([hi, lo]), np.concatenate([w, w]))


def rgg_sizes(count: int = 48, lo: int = 1024, hi: int = 65536, seed: int = 7) -> list[int]:
    """Vertex counts drawn log-uniformly in [lo, hi]."""
    u = rand_unit(seed, 99, np.arange(count, dtype=np.int64))
    return [int(round(math.exp(math.log(lo) + t * (math.log(hi) - math.log(lo))))) for t in u]


def rgg_batch(count: int = 48, seed: int = 7) -> list[EdgeList]:
    """The multi-graph batch: ``count`` random geometric 3-NN graphs."""
    return [rgg_knn(nv, seed=seed, gid=g) for g, nv in enumerate(rgg_sizes(count, seed=seed))]


WORKLOADS = {
    "grid32": lambda: road_grid(32, 32, drop=0.0, highway=0.0),
    "grid256": lambda: road_grid(256, 256),
    "grid512": lambda: road_grid(512, 512),
    "grid2048": lambda: road_grid(2048, 2048, highway=0.001, radius=128),
}

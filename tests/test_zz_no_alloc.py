"""fbc_single_source_noalloc: the entry point for callers that cannot allocate device memory.

Callers inside a framework's memory pool, behind a custom allocator that owns every device
byte, or handed device buffers and a stream by their host application cannot let the
library call cudaMalloc.  This entry point takes the graph and the output as the caller's
device buffers and keeps its work area in a fixed device array inside the library.  The tests
hand it device buffers (allocated here by PyTorch, standing in for such a caller) through the
C ABI and check its results against fbc_single_source, the existing entry point, within the
tolerances of the other parity tests: two calls in a row on the 256x256 grid, a small graph
right after the large one (the shared array keeps the previous call's contents), a unit-weight
grid whose path counts pass 2^64 (the FP64-count rerun), and the error paths (malformed CSR,
distance range, sizes beyond the work area), each followed by a good call.
"""
import ctypes as C

import numpy as np
import pytest

import graphs

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-9
TOL_FP32C = 1e-6
MAX_N = 262144


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.abs(a - b)
    d[(a == 0) & (b == 0)] = 0
    return float(np.max(d / np.maximum(np.abs(b), 1e-300)))


def _entry(fg):
    f = fg.lib.fbc_single_source_noalloc
    f.argtypes = [C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_int32, C.c_int, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


class DevCSR:
    """A caller's device buffers: int32 row offsets, (destination, weight) int32 pairs, output."""

    def __init__(self, rp, col, w):
        import torch

        dev = torch.device("cuda", 0)
        self.n = rp.size - 1
        self.m = int(rp[-1])
        self.rp = torch.from_numpy(np.ascontiguousarray(rp, np.int32)).to(dev)
        adj = np.stack([np.asarray(col, np.int64), np.asarray(w, np.int64)], axis=1).astype(np.int32)
        self.adj = torch.from_numpy(np.ascontiguousarray(adj.ravel() if adj.size else np.zeros(2, np.int32))).to(dev)
        self.dep = torch.empty(self.n, dtype=torch.float64, device=dev)

    def call(self, f, src, prec, m=None):
        import torch

        self.dep.fill_(-1.0)  # the entry point must overwrite every entry
        torch.cuda.synchronize()
        return f(self.n, self.m if m is None else m, self.rp.data_ptr(), self.adj.data_ptr(), src, prec,
                 self.dep.data_ptr(), None)


def _check(fg, f, dc, g, src, prec, tol):
    rc = dc.call(f, src, prec)
    assert rc == fg.FBC_OK, fg.lib.fbc_last_error_string()
    got = dc.dep.cpu().numpy()
    want = fg.single_source(g, src, prec)
    assert got[src] == 0.0
    assert rel_err(got, want) <= tol


def unit_grid(k):
    """k x k 4-neighbour grid, both directions, all weights 1: from a corner, the far corner has
    C(2k-2, k-1) shortest paths (above 2^64 for k >= 35)."""
    src, dst = [], []
    for r in range(k):
        for c in range(k):
            v = r * k + c
            for dr, dc in ((-1, 0), (0, -1), (0, 1), (1, 0)):
                rr, cc = r + dr, c + dc
                if 0 <= rr < k and 0 <= cc < k:
                    src.append(v)
                    dst.append(rr * k + cc)
    src, dst = np.array(src), np.array(dst)
    o = np.lexsort((dst, src))
    src, dst = src[o], dst[o]
    rp = np.zeros(k * k + 1, np.int64)
    rp[1:] = np.cumsum(np.bincount(src, minlength=k * k))
    return rp, dst.astype(np.int32), np.ones(dst.size, np.int32)


def test_noalloc_matches_single_source(fg):
    pytest.importorskip("torch")
    el = graphs.WORKLOADS["grid256"]()
    rp, col, w = el.csr()
    g = fg.Graph.from_edgelist(el)
    dc = DevCSR(rp, col, w)
    f = _entry(fg)
    for prec, tol, src in ((fg.FP64, TOL_FP64, 17), (fg.FP64, TOL_FP64, 40000), (fg.FP32C, TOL_FP32C, 123)):
        _check(fg, f, dc, g, src, prec, tol)
    # a small graph right after the large one: the shared array still holds the last call's state
    el2 = graphs.road_grid(12, 12, seed=5)
    rp2, col2, w2 = el2.csr()
    dc2 = DevCSR(rp2, col2, w2)
    g2 = fg.Graph.from_edgelist(el2)
    for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
        _check(fg, f, dc2, g2, 0, prec, tol)
        _check(fg, f, dc2, g2, 77, prec, tol)


def test_noalloc_path_counts_beyond_64_bits(fg):
    """The far corner of a 35x35 unit grid has C(68, 34) ~ 2.8e19 > 2^64 shortest paths: the
    entry point reruns the source with FP64 counts, as fbc_single_source does."""
    pytest.importorskip("torch")
    import oracle

    rp, col, w = unit_grid(35)
    g = fg.Graph.from_csr(rp, col, w.astype(np.float64))
    dc = DevCSR(rp, col, w)
    f = _entry(fg)
    for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
        _check(fg, f, dc, g, 0, prec, tol)
    # and against the oracle (double path counts, as the reference keeps them)
    rc = dc.call(f, 0, fg.FP64)
    assert rc == fg.FBC_OK, fg.lib.fbc_last_error_string()
    want = oracle.single_source(oracle.CSR(rp, col, w.astype(np.float64)), 0)
    assert rel_err(dc.dep.cpu().numpy(), want) <= TOL_FP64


def test_noalloc_rejects_malformed_csr(fg):
    pytest.importorskip("torch")
    el = graphs.road_grid(12, 12, seed=5)
    rp, col, w = el.csr()
    g = fg.Graph.from_edgelist(el)
    f = _entry(fg)
    bad_id = col.copy()
    bad_id[5] = el.n  # destination out of range
    bad_w = w.copy()
    bad_w[7] = 0  # weight <= 0
    unsorted = col.copy()
    a = int(np.argmax(np.diff(rp) >= 2))  # a row with two edges: swap them
    unsorted[rp[a]], unsorted[rp[a] + 1] = col[rp[a] + 1], col[rp[a]]
    for c, ww in ((bad_id, w), (col, bad_w), (unsorted, w)):
        dc = DevCSR(rp, c, ww)
        assert dc.call(f, 0, fg.FP64) == fg.FBC_ERR_INVALID_ARG
        assert b"malformed" in fg.lib.fbc_last_error_string()
    dc = DevCSR(rp, col, w)
    # the caller's edge count disagrees with row_ptr[n] (rows then reach past the given buffer)
    assert dc.call(f, 0, fg.FP64, m=dc.m - 1) == fg.FBC_ERR_INVALID_ARG
    assert dc.call(f, 0, fg.FP64, m=-1) == fg.FBC_ERR_INVALID_ARG
    assert dc.call(f, el.n, fg.FP64) == fg.FBC_ERR_INVALID_ARG  # source out of range
    _check(fg, f, dc, g, 3, fg.FP64, TOL_FP64)  # a good call after the rejected ones


def test_noalloc_rejects_distance_range(fg):
    """n * max_weight beyond the int32 distance range: FBC_ERR_RANGE, as the other entry points."""
    pytest.importorskip("torch")
    el = graphs.road_grid(12, 12, seed=5)
    rp, col, w = el.csr()
    w2 = w.copy()
    w2[3] = 20_000_000  # 144 * 2e7 > 2^31
    dc = DevCSR(rp, col, w2)
    f = _entry(fg)
    assert dc.call(f, 0, fg.FP64) == fg.FBC_ERR_RANGE
    g = fg.Graph.from_edgelist(el)
    _check(fg, f, DevCSR(rp, col, w), g, 5, fg.FP32C, TOL_FP32C)


def test_noalloc_rejects_sizes_beyond_its_work_area(fg):
    f = _entry(fg)
    rc = f(MAX_N + 1, 0, C.c_void_p(16), C.c_void_p(16), 0, fg.FP64, C.c_void_p(16), None)
    assert rc == fg.FBC_ERR_RANGE
    assert b"262144" in fg.lib.fbc_last_error_string()

"""fbc_single_source_noalloc: the entry point for callers that cannot allocate device memory.

Callers inside a framework's memory pool, behind a custom allocator that owns every device
byte, or handed device buffers and a stream by their host application cannot let the
library call cudaMalloc.  This entry point takes the graph and the output as the caller's
device buffers and keeps its work area in a fixed device array inside the library.  The test
hands it device buffers (allocated here by PyTorch, standing in for such a caller) through
the C ABI and checks two calls in a row against fbc_single_source, the existing entry point,
within the tolerances of the other parity tests.
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
    f.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_int, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_matches_single_source(fg):
    torch = pytest.importorskip("torch")
    el = graphs.WORKLOADS["grid256"]()
    rp, col, w = el.csr()
    g = fg.Graph.from_edgelist(el)
    dev = torch.device("cuda", 0)
    d_rp = torch.from_numpy(rp.astype(np.int32)).to(dev)
    d_adj = torch.from_numpy(np.stack([col, w], axis=1).astype(np.int32).ravel()).to(dev)
    d_dep = torch.empty(el.n, dtype=torch.float64, device=dev)
    f = _entry(fg)
    for prec, tol, src in ((fg.FP64, TOL_FP64, 17), (fg.FP64, TOL_FP64, 40000), (fg.FP32C, TOL_FP32C, 123)):
        d_dep.fill_(-1.0)  # the entry point must overwrite every entry
        torch.cuda.synchronize()
        rc = f(el.n, d_rp.data_ptr(), d_adj.data_ptr(), src, prec, d_dep.data_ptr(), None)
        assert rc == fg.FBC_OK, fg.lib.fbc_last_error_string()
        got = d_dep.cpu().numpy()
        want = fg.single_source(g, src, prec)
        assert got[src] == 0.0
        assert rel_err(got, want) <= tol


def test_noalloc_rejects_sizes_beyond_its_work_area(fg):
    f = _entry(fg)
    rc = f(MAX_N + 1, C.c_void_p(16), C.c_void_p(16), 0, fg.FP64, C.c_void_p(16), None)
    assert rc == fg.FBC_ERR_RANGE
    assert b"262144" in fg.lib.fbc_last_error_string()

"""Batched runs on graphs of at least `order_min_n` vertices use a relabelled copy of the CSR
(recursive BFS bisection, for memory locality) and map their outputs back to the input ids.
With the threshold at 0 every batched whole-graph run takes that path: results must match the
oracle as in the input order."""
import numpy as np
import pytest

import graphs
import oracle
from test_gpu_parity import TOL_FP32C, TOL_FP64, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture
def relabel_all(fg):
    old = fg.get_option("order_min_n")
    fg.set_option("order_min_n", 0)
    yield
    fg.set_option("order_min_n", old)


def test_exact_bc_relabelled(fg, relabel_all):
    el = graphs.WORKLOADS["grid32"]()
    g = fg.Graph.from_edgelist(el)
    ref = oracle.exact_bc(oracle.CSR.from_edgelist(el))
    for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
        assert rel_err(fg.exact_bc(g, prec, fg.BATCHED), ref) <= tol


def test_pivot_batch_relabelled(fg, relabel_all):
    el = graphs.WORKLOADS["grid256"]()
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    rng = np.random.default_rng(9)
    piv = rng.choice(el.n, 40, replace=False).astype(np.int32)
    cards = rng.integers(1, 9, piv.size).astype(np.float64)
    ref = oracle.pivot_batch(og, piv, cards)
    for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
        assert rel_err(fg.dependency_batch(g, piv, cards, prec, fg.BATCHED), ref) <= tol


def test_multi_graph_relabelled(fg, relabel_all):
    """Several graphs in one launch: each relabelled graph writes through its own offset."""
    els = [graphs.rgg_knn(n, seed=5, gid=i) for i, n in enumerate([1024, 1300, 2100])]
    gs = [fg.Graph.from_edgelist(e) for e in els]
    fg.set_option("warp_max_n", 0)  # every graph on the frontier kernel
    try:
        outs = fg.multi_exact_bc(gs, fg.FP64, fg.BATCHED)
    finally:
        fg.set_option("warp_max_n", 4096)
    for e, o in zip(els, outs):
        assert rel_err(o, oracle.exact_bc(oracle.CSR.from_edgelist(e))) <= TOL_FP64

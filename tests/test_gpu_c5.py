"""Parity on the full-form workload: the 2048x2048 road grid (4,194,304 vertices, 15.9M edges)
with the reference's own Louvain partition (seeds 1-4, precision 0.01; the communities of
tests/golden/grid2048_partition.npz).

* Clusters: the largest community (25,916 vertices) and two of median size run through
  fbc_cluster_eval_batch in the batched schedule -- the frontier kernel with four sources per
  block, interleaved state and wide rows, the path the clustered bench takes for these clusters
  -- against the oracle's cluster evaluation (DijkstraClusterEvaluator.h:50-180): intra-cluster
  BC within 1e-9 (FP64) / 1e-6 (FP32C), border lengths and counts bit-exact.
* Pivots: 16 pivots over the whole graph through fbc_sssp_dependency_batch (the locality-ordered
  copy of the graph, wide blocks) against the oracle's pivot batch (DijkstraSSBrandesBC.h:45-81
  weighted by class cardinality, ClusteredBrandesBC.h:141-155).
"""
import os

import numpy as np
import pytest

import graphs
import oracle
from conftest import GOLDEN
from test_gpu_parity import TOL_FP32C, TOL_FP64, rel_err

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def c5(fg):
    el = graphs.WORKLOADS["grid2048"]()
    cid = np.load(os.path.join(GOLDEN, "grid2048_partition.npz"))["community"].astype(np.int64)
    order = np.argsort(cid, kind="stable").astype(np.int32)
    off = np.zeros(int(cid.max()) + 2, np.int64)
    off[1:] = np.cumsum(np.bincount(cid))
    g = fg.Graph.from_edgelist(el)
    og = oracle.CSR.from_edgelist(el)
    return el, g, og, order, off


def _clusters(off, order):
    sizes = np.diff(off)
    by = np.argsort(sizes, kind="stable")
    big = int(by[-1])
    med = [int(by[by.size // 2]), int(by[by.size // 2 + 1])]
    return [big] + med


def test_c5_clusters_match_oracle(fg, c5):
    el, g, og, order, off = c5
    picks = _clusters(off, order)
    clusters = [order[off[c]:off[c + 1]] for c in picks]
    assert clusters[0].size == 25916
    cs = fg.ClusterSet.from_lists(clusters).with_borders(g)
    ref_bc = np.zeros(el.n)
    refs = []
    for c, vs in enumerate(clusters):
        b = cs.borders[cs.boff[c]:cs.boff[c + 1]]
        assert b.size > 0
        _, bd, bs = oracle.cluster_eval(og, vs, b, ref_bc, threads=THREADS)
        refs.append((bd, bs))
    members = np.concatenate(clusters)
    for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
        st = fg.Stats()
        ev = fg.cluster_eval_batch(g, cs, prec, fg.BATCHED, stats=st)
        assert st.group == 4 and st.warp_units == 0  # the grouped frontier path
        assert rel_err(ev.intra_bc[members], ref_bc[members]) <= tol
        assert np.all(ev.intra_bc[np.setdiff1d(np.arange(el.n), members)] == 0)
        for c, (bd, bs) in enumerate(refs):
            e0, e1 = ev.entry_off[c], ev.entry_off[c + 1]
            nb = bd.shape[1]
            assert np.array_equal(ev.border_dist[e0:e1].reshape(-1, nb), bd)
            assert np.array_equal(ev.border_sigma[e0:e1].reshape(-1, nb).astype(np.float64), bs)


def test_c5_cluster_plan_captured(fg, c5):
    """The same three communities as a prepared sweep: the frontier-kernel launch is captured, and
    every replay equals the direct batched evaluation (border vectors bit-exact, intra BC within the
    precision form's bound)."""
    el, g, og, order, off = c5
    picks = _clusters(off, order)
    cs = fg.ClusterSet.from_lists([order[off[c]:off[c + 1]] for c in picks]).with_borders(g)
    for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
        base = fg.cluster_eval_batch(g, cs, prec, fg.BATCHED)
        plan = fg.ClusterPlan(g, cs, prec)
        assert plan.captured
        for _ in range(2):
            st = fg.Stats()
            ev = plan.run(st)
            assert st.launches == 1 and st.block_units == cs.vertices.size
            assert rel_err(ev.intra_bc, base.intra_bc) <= tol
            assert np.array_equal(ev.border_dist, base.border_dist)
            assert np.array_equal(ev.border_sigma, base.border_sigma)
        plan.free()


def test_c5_pivots_match_oracle(fg, c5):
    el, g, og, order, off = c5
    src = np.unique(graphs.rand_int(23, 5, np.arange(16), 0, el.n - 1)).astype(np.int32)
    cards = (1 + graphs.rand_int(23, 6, np.arange(src.size), 0, 40)).astype(np.float64)
    ref = oracle.pivot_batch(og, src, cards, threads=THREADS)
    for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
        st = fg.Stats()
        got = fg.dependency_batch(g, src, cards, prec, fg.BATCHED, stats=st)
        assert st.block_units == src.size and st.retries == 0
        assert rel_err(got, ref) <= tol

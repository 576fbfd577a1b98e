"""Edge cases the reference's code paths meet: graphs without edges, isolated and unreachable
vertices, single-vertex clusters (no borders), clusters without intra-cluster edges, sources with
nothing reachable -- for both schedules and both precisions."""
import numpy as np
import pytest

import graphs
import oracle
from test_gpu_parity import TOL_FP32C, TOL_FP64, rel_err

pytestmark = pytest.mark.gpu
FORMS = [(0, 0), (0, 1), (1, 1)]  # (precision, schedule)


def _chain_with_island():
    # 0 -> 1 -> 2 -> 3 (a chain), 5 <-> 6 (an island), 4 isolated: n = 7 (1 + max source 6)
    src = np.array([0, 1, 2, 5, 6], np.int32)
    dst = np.array([1, 2, 3, 6, 5], np.int32)
    w = np.array([2.0, 3.0, 1.0, 4.0, 4.0])
    return src, dst, w


@pytest.mark.parametrize("prec,sched", FORMS)
def test_unreachable_and_isolated(fg, prec, sched):
    src, dst, w = _chain_with_island()
    g = fg.Graph.from_edges(src, dst, w)
    assert g.n == 7
    og = oracle.CSR(*g.csr())
    tol = TOL_FP64 if prec == 0 else TOL_FP32C
    assert rel_err(fg.exact_bc(g, prec, sched), oracle.exact_bc(og)) <= tol
    # a source that reaches nothing, and an isolated one
    for s in (3, 4):
        d = fg.dependency_batch(g, np.array([s], np.int32), None, prec, sched)
        assert np.all(d == 0)


@pytest.mark.parametrize("prec,sched", FORMS)
def test_empty_source_list_and_single_vertex(fg, prec, sched):
    el = graphs.WORKLOADS["grid32"]()
    g = fg.Graph.from_edgelist(el)
    out = fg.dependency_batch(g, np.zeros(0, np.int32), None, prec, sched)
    assert out.shape == (el.n,) and np.all(out == 0)
    g1 = fg.Graph.from_edges(np.array([0], np.int32), np.array([0], np.int32), np.array([1.0]))
    assert g1.n == 1 and np.all(fg.exact_bc(g1, prec, sched) == 0)


@pytest.mark.parametrize("prec,sched", FORMS)
def test_degenerate_clusters(fg, prec, sched):
    """Single-vertex clusters (no intra edges) and a cluster whose vertices share no edge: their
    intra BC is 0 and every border vector is (0, 0) except a vertex's own entry (0, 1)."""
    el = graphs.road_grid(16, 16, seed=5)
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    ids = np.arange(el.n)
    singles = [np.array([v], np.int32) for v in (0, 17, 255)]
    scattered = np.array([2, 40, 100, 200], np.int32)   # pairwise non-adjacent on the grid
    rest = np.setdiff1d(ids, np.concatenate(singles + [scattered])).astype(np.int32)
    clusters = singles + [scattered, rest]
    cs = fg.ClusterSet.from_lists(clusters).with_borders(g)
    ev = fg.cluster_eval_batch(g, cs, prec, sched)
    ref_bc = np.zeros(el.n)
    for c, vs in enumerate(clusters):
        b = cs.borders[cs.boff[c]:cs.boff[c + 1]]
        _, bd, bs = oracle.cluster_eval(og, vs, b, ref_bc)
        for i in range(0, vs.size, max(1, vs.size // 7)):
            L, Cn = ev.vertex_info(c, i)
            assert np.array_equal(L, bd[i]) and np.array_equal(Cn.astype(np.float64), bs[i])
    tol = TOL_FP64 if prec == 0 else TOL_FP32C
    assert rel_err(ev.intra_bc, ref_bc) <= tol
    for vs in singles + [scattered]:
        assert np.all(ev.intra_bc[vs] == 0)

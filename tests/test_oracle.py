"""The CPU oracle pinned to the reference's known answers (CPU only)."""
import os

import numpy as np
import pytest

import graphs
import oracle
from conftest import GOLDEN


def dwg_csr():
    a = np.loadtxt(os.path.join(GOLDEN, "DWGtext.txt"), ndmin=2)
    s, d, w = a[:, 0].astype(np.int32), a[:, 1].astype(np.int32), a[:, 2]
    n = int(s.max()) + 1
    o = np.lexsort((d, s))
    rp = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(s[o], minlength=n), out=rp[1:])
    return oracle.CSR(rp, d[o], w[o])


def sub_csr(g, verts):
    """Induced subgraph on ids 0..k-1 (the reference's SubGraph {0..4} test fixture)."""
    k = len(verts)
    rows, cols, ws = [], [], []
    rp = [0]
    for v in verts:
        for e in range(g.rp[v], g.rp[v + 1]):
            if g.col[e] < k:
                cols.append(g.col[e]); ws.append(g.w[e])
        rp.append(len(cols))
    return oracle.CSR(np.array(rp), np.array(cols, np.int32), np.array(ws))


def test_exact_subgraph_known_answer():
    """libfastbc/test/brandes/ExactBrandesBC.cpp:31-35."""
    bc = oracle.exact_bc(sub_csr(dwg_csr(), [0, 1, 2, 3, 4]))
    assert list(bc) == [2.0, 2.0, 0.5, 1.0, 0.0]


def test_cluster_evaluator_known_answers():
    """libfastbc/test/brandes/DijkstraClusterEvaluator.cpp:38-74."""
    g = dwg_csr()
    bc, bd, bs = oracle.cluster_eval(g, [0, 1, 2, 3, 4], [3, 4])
    assert list(bc) == [2, 2, 0.5, 1, 0, 0, 0, 0, 0]
    want_len = [[5, 7], [1, 4], [8, 4], [0, 3], [0, 0]]
    want_cnt = [[1, 2], [1, 1], [1, 1], [1, 1], [0, 1]]
    assert bd.tolist() == want_len and bs.tolist() == want_cnt


def test_full_dwg_exact_golden():
    """Reference ExactBrandesBC<int,double> on the whole test graph (golden from the reference)."""
    bc = oracle.exact_bc(dwg_csr())
    golden = [2, 4.333333333333333, 1.3333333333333333, 7.333333333333333,
              7.6666666666666661, 7.333333333333333, 0, 0, 2]
    assert bc.tolist() == golden


def test_grid32_exact_matches_reference_bitwise():
    path = os.path.join(GOLDEN, "grid32_exact_bc.txt")
    golden = np.loadtxt(path)
    bc = oracle.exact_bc(oracle.CSR.from_edgelist(graphs.WORKLOADS["grid32"]()))
    assert np.array_equal(bc, golden)


def test_grid32_threads_agree():
    g = oracle.CSR.from_edgelist(graphs.WORKLOADS["grid32"]())
    a = oracle.exact_bc(g, 1)
    b = oracle.exact_bc(g, 4)
    assert np.max(np.abs(a - b) / np.maximum(a, 1e-300)) < 1e-12


def test_single_source_and_dump_consistent():
    g = oracle.CSR.from_edgelist(graphs.WORKLOADS["grid32"]())
    dep = oracle.single_source(g, 77)
    dist, sig, dlt, order, preds = oracle.sssp_dump(g, 77)
    assert dep[77] == 0
    assert np.array_equal(dep[np.arange(g.n) != 77], dlt[np.arange(g.n) != 77])
    assert order[0] == 77 and np.all(np.diff(dist[order]) >= 0)
    for v in range(g.n):
        assert sig[v] == sum(sig[p] for p in preds[v]) or v == 77


def test_grid32_single_source_matches_reference():
    z = np.load(os.path.join(GOLDEN, "grid32_ss.npz"))
    g = oracle.CSR.from_edgelist(graphs.WORKLOADS["grid32"]())
    for s, dep in zip(z["sources"], z["dep"]):
        assert np.array_equal(oracle.single_source(g, int(s)), dep)


def test_grid256_clusters_match_reference_intra_bc():
    """DijkstraClusterEvaluator on the reference's own Louvain clusters: bit-identical."""
    z = np.load(os.path.join(GOLDEN, "grid256_clustered.npz"))
    g = oracle.CSR.from_edgelist(graphs.WORKLOADS["grid256"]())
    off, cv, boff, bv = z["cluster_off"], z["cluster_vertices"], z["border_off"], z["borders"]
    acc = np.zeros(g.n)
    for c in (0, 7, 33):
        vs = cv[off[c]:off[c + 1]]
        oracle.cluster_eval(g, vs, bv[boff[c]:boff[c + 1]], acc)
        assert np.array_equal(acc[vs], z["intra_bc"][vs])


def test_generators_are_stable():
    """The seeded generators are part of the workload definition."""
    el = graphs.WORKLOADS["grid256"]()
    assert (el.n, el.m) == (65536, 248528)
    assert int(el.w.sum()) == 12506652
    assert graphs.WORKLOADS["grid32"]().m == 3968
    assert graphs.rgg_sizes()[:3] == [1765, 2433, 1422]


def test_rgg_exact_matches_reference_bitwise():
    """A 1,500-point random geometric graph (3-NN, weights ceil(1000 d); the 48-graph batch's
    family): the oracle's exact BC equals the reference's, bit for bit."""
    golden = np.loadtxt(os.path.join(GOLDEN, "rgg1500_exact_bc.txt"))
    bc = oracle.exact_bc(oracle.CSR.from_edgelist(graphs.rgg_knn(1500, seed=11)))
    assert np.array_equal(bc, golden)


def test_rgg_single_source_matches_reference_bitwise():
    """DijkstraSSBrandesBC::singleSourceBrandes on the same graph for three sources."""
    z = np.load(os.path.join(GOLDEN, "rgg1500_ss.npz"))
    g = oracle.CSR.from_edgelist(graphs.rgg_knn(1500, seed=11))
    for s, dep in zip(z["sources"], z["dep"]):
        assert np.array_equal(oracle.single_source(g, int(s)), dep)


def test_rgg_cluster_matches_reference_bitwise():
    """DijkstraClusterEvaluator on a scattered cluster of the same graph (489 of its 500 members
    are borders, many unreachable from a member): intra BC and every border (length, count)."""
    z = np.load(os.path.join(GOLDEN, "rgg1500_cluster.npz"))
    g = oracle.CSR.from_edgelist(graphs.rgg_knn(1500, seed=11))
    bc, bd, bs = oracle.cluster_eval(g, np.arange(500, dtype=np.int32), z["borders"])
    assert np.array_equal(bc, z["intra_bc"])
    assert np.array_equal(bd, z["border_len"]) and np.array_equal(bs, z["border_cnt"])


def _grid256_kmeans_inputs(clusters):
    el = graphs.WORKLOADS["grid256"]()
    og = oracle.CSR.from_edgelist(el)
    z = np.load(os.path.join(GOLDEN, "grid256_clustered.npz"))
    zc = np.load(os.path.join(GOLDEN, "grid256_classes.npz"))
    off, cv, boff, bv = z["cluster_off"], z["cluster_vertices"], z["border_off"], z["borders"]
    for c in clusters:
        vs, bs = cv[off[c]:off[c + 1]], bv[boff[c]:boff[c + 1]]
        _, bd, bsg = oracle.cluster_eval(og, vs, bs, None, threads=4)
        pos = {int(v): i for i, v in enumerate(vs)}
        cls = zc["pivots"][zc["class_off"][c]:zc["class_off"][c + 1]]
        crd = zc["cards"][zc["class_off"][c]:zc["class_off"][c + 1]]
        rows = np.array([pos[int(v)] for v in cls])
        L = bd[rows] - bd[rows].min(axis=1, keepdims=True)  # VertexInfo::normalize
        yield c, cls, crd, L, bsg[rows].astype(np.int64).astype(np.int32), z


def test_kmeans_matches_reference_pivot_sets():
    """The k-means step (PlusPlusKMeans + KMeansPivotSelector, kfrac 0.5) restated in the oracle
    gives the reference's own pivot set and weights, bit for bit, on 12 of the 256x256 grid's
    Louvain communities (all 76 agree too; 12 keep the CPU suite short): exact classes from the
    reference's selector, border vectors from the oracle's cluster evaluation."""
    z = np.load(os.path.join(GOLDEN, "grid256_clustered.npz"))
    with_borders = [c for c in range(z["cluster_off"].size - 1) if z["border_off"][c + 1] > z["border_off"][c]]
    for c, cls, crd, L, Cn, z in _grid256_kmeans_inputs(with_borders[::6]):
        idx, w = oracle.kmeans_pivots(L, Cn, crd)
        p0, p1 = z["pivot_off"][c], z["pivot_off"][c + 1]
        assert np.array_equal(cls[idx], z["pivots"][p0:p1]), f"community {c}"
        assert np.array_equal(w, z["cards"][p0:p1]), f"community {c}"
        assert int(w.sum()) == int(crd.sum())

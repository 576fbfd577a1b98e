"""GPU parity through the C ABI (libfbcgpu.so) against the CPU oracle.

Bars (the engine's contract):
  * distances and shortest-path counts bit-exact; predecessor sets equal (the oracle's
    predecessor lists, compared as sets with the tight in-edges implied by the GPU distances);
  * BC within 1e-9 relative of the FP64 oracle in the plain (FP64) form;
  * BC within 1e-6 relative in the FP32-compensated form.
"""
import numpy as np
import pytest

import graphs
import oracle

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-9
TOL_FP32C = 1e-6


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.maximum(np.abs(b), 1e-300)
    d = np.abs(a - b)
    d[(a == 0) & (b == 0)] = 0
    return float(np.max(d / scale)) if d.size else 0.0


def dwg():
    import os
    from conftest import GOLDEN

    a = np.loadtxt(os.path.join(GOLDEN, "DWGtext.txt"), ndmin=2)
    return a[:, 0].astype(np.int32), a[:, 1].astype(np.int32), a[:, 2]


def to_csr(src, dst, w):
    n = int(src.max()) + 1
    order = np.lexsort((dst, src))
    s, d, ww = src[order], dst[order], w[order]
    rp = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(s, minlength=n), out=rp[1:])
    return oracle.CSR(rp, d, ww)


def check_source(fg, g, og, src):
    dist, sig, dlt, npred = fg.sssp_debug(g, src)
    od, osg, odl, order, preds = oracle.sssp_dump(og, src)
    gd = np.where(dist < 0, np.inf, dist.astype(np.float64))
    assert np.array_equal(gd, od), f"dist differs for source {src}"
    assert np.array_equal(sig.astype(np.float64), osg), f"sigma differs for source {src}"
    assert np.array_equal(npred, np.array([len(p) for p in preds])), f"pred count differs, source {src}"
    # predecessor sets: the oracle's lists equal the tight in-edges implied by the GPU distances,
    # for every vertex (pairs (v, x) encoded as x * n + v)
    rp, col, w = og.rp, og.col, og.w
    n = rp.size - 1
    tail = np.repeat(np.arange(n, dtype=np.int64), np.diff(rp))
    tight = np.isfinite(gd[tail]) & (gd[tail] + w == gd[col])
    got_pairs = col[tight].astype(np.int64) * n + tail[tight]
    lens = np.array([len(p) for p in preds])
    ora_pairs = np.repeat(np.arange(n, dtype=np.int64), lens) * n + (
        np.concatenate(preds).astype(np.int64) if lens.sum() else np.zeros(0, np.int64))
    assert got_pairs.size == ora_pairs.size
    assert np.array_equal(np.sort(got_pairs), np.sort(ora_pairs)), f"predecessor sets differ for source {src}"
    reached = od < np.inf
    assert rel_err(dlt[reached], odl[reached]) <= TOL_FP64


def test_dwg_sssp_bit_exact(fg):
    s, d, w = dwg()
    g = fg.Graph.from_edges(s, d, w)
    og = to_csr(s, d, w)
    assert g.n == 9 and g.m == 16
    for src in range(9):
        check_source(fg, g, og, src)


def test_dwg_exact_bc_matches_reference_golden(fg):
    """Full-graph exact BC of the reference's test graph (reference ExactBrandesBC, FP64)."""
    s, d, w = dwg()
    g = fg.Graph.from_edges(s, d, w)
    golden = np.array([2, 4.333333333333333, 1.3333333333333333, 7.333333333333333,
                       7.6666666666666661, 7.333333333333333, 0, 0, 2])
    for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
        for sched in (fg.PLAIN, fg.BATCHED):
            bc = fg.exact_bc(g, prec, sched)
            assert rel_err(bc, golden) <= tol


def test_dwg_subgraph_known_answers(fg):
    """ExactBrandesBC.cpp:31-35 and DijkstraClusterEvaluator.cpp:38-74 on SubGraph {0..4}."""
    s, d, w = dwg()
    g = fg.Graph.from_edges(s, d, w)
    cs = fg.ClusterSet.from_lists([[0, 1, 2, 3, 4]])
    for prec in (fg.FP64, fg.FP32C):
        for sched in (fg.PLAIN, fg.BATCHED):
            ev = fg.cluster_eval_batch(g, cs, prec, sched)
            assert np.array_equal(ev.intra_bc, [2, 2, 0.5, 1, 0, 0, 0, 0, 0])
            assert list(ev.clusters.borders) == [3, 4]
            want = {0: ([5, 7], [1, 2]), 1: ([1, 4], [1, 1]), 2: ([8, 4], [1, 1]),
                    3: ([0, 3], [1, 1]), 4: ([0, 0], [0, 1])}
            for i, (lens, cnts) in want.items():
                L, Cn = ev.vertex_info(0, i)
                assert list(L) == lens and list(Cn) == cnts


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("sched", [0, 1])
def test_grid32_exact(fg, prec, sched):
    el = graphs.WORKLOADS["grid32"]()
    og = oracle.CSR.from_edgelist(el)
    ref = oracle.exact_bc(og)
    g = fg.Graph.from_edgelist(el)
    bc = fg.exact_bc(g, prec, sched)
    assert rel_err(bc, ref) <= (TOL_FP64 if prec == 0 else TOL_FP32C)


def test_grid32_sources_bit_exact(fg):
    el = graphs.WORKLOADS["grid32"]()
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    for src in (0, 1, 31, 500, 1023):
        check_source(fg, g, og, src)


def test_grid256_sources_bit_exact(fg):
    el = graphs.WORKLOADS["grid256"]()
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    for src in (0, 12345, 65535):
        check_source(fg, g, og, src)


@pytest.mark.parametrize("prec", [0, 1])
def test_grid256_pivot_batch(fg, prec):
    el = graphs.WORKLOADS["grid256"]()
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    rng = np.random.default_rng(3)
    piv = rng.choice(el.n, 24, replace=False).astype(np.int32)
    cards = rng.integers(1, 9, piv.size).astype(np.float64)
    ref = oracle.pivot_batch(og, piv, cards)
    for sched in (fg.PLAIN, fg.BATCHED):
        got = fg.dependency_batch(g, piv, cards, prec, sched)
        assert rel_err(got, ref) <= (TOL_FP64 if prec == 0 else TOL_FP32C)


def test_rgg_small_exact(fg):
    """The oracle's exact BC here equals the reference's bit for bit (tests/golden/
    rgg1500_exact_bc.txt, pinned in tests/test_oracle.py)."""
    import os
    from conftest import GOLDEN

    el = graphs.rgg_knn(1500, seed=11)
    og = oracle.CSR.from_edgelist(el)
    ref = oracle.exact_bc(og)
    assert np.array_equal(ref, np.loadtxt(os.path.join(GOLDEN, "rgg1500_exact_bc.txt")))
    g = fg.Graph.from_edgelist(el)
    for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
        for sched in (fg.PLAIN, fg.BATCHED):
            assert rel_err(fg.exact_bc(g, prec, sched), ref) <= tol
    for src in (0, 700, 1499):
        check_source(fg, g, og, src)


def test_multi_graph_batch(fg):
    els = [graphs.rgg_knn(n, seed=5, gid=i) for i, n in enumerate([1024, 1300, 2100])]
    gs = [fg.Graph.from_edgelist(e) for e in els]
    for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
        outs = fg.multi_exact_bc(gs, prec, fg.BATCHED)
        for e, o in zip(els, outs):
            assert rel_err(o, oracle.exact_bc(oracle.CSR.from_edgelist(e))) <= tol


def test_cluster_eval_grid(fg):
    """Tile a 64x64 grid into 16 square clusters; compare intra BC and border (dist, sigma)."""
    el = graphs.road_grid(64, 64, seed=9)
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    ids = np.arange(el.n)
    tile = (ids // 64) // 16 * 4 + (ids % 64) // 16
    clusters = [ids[tile == t].astype(np.int32) for t in range(16)]
    cs = fg.ClusterSet.from_lists(clusters).with_borders(g)
    ref_bc = np.zeros(el.n)
    refs = []
    for c, vs in enumerate(clusters):
        b = cs.borders[cs.boff[c]:cs.boff[c + 1]]
        _, bd, bs = oracle.cluster_eval(og, vs, b, ref_bc)
        refs.append((bd, bs))
    for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
        for sched in (fg.PLAIN, fg.BATCHED):
            ev = fg.cluster_eval_batch(g, cs, prec, sched)
            assert rel_err(ev.intra_bc, ref_bc) <= tol
            for c, (bd, bs) in enumerate(refs):
                for i in range(len(clusters[c])):
                    L, Cn = ev.vertex_info(c, i)
                    assert np.array_equal(L, bd[i]) and np.array_equal(Cn.astype(np.float64), bs[i])


def test_invalid_inputs_raise(fg):
    with pytest.raises(fg.FbcError) as e:
        fg.Graph.from_edges(np.array([0, 1], np.int32), np.array([1, 0], np.int32), np.array([1.0, 0.0]))
    assert e.value.code == fg.FBC_ERR_INVALID_ARG
    with pytest.raises(fg.FbcError):
        fg.Graph.from_edges(np.array([0], np.int32), np.array([5], np.int32), np.array([1.0]))
    with pytest.raises(fg.FbcError) as e:
        fg.Graph.from_edges(np.array([0, 1], np.int32), np.array([1, 0], np.int32), np.array([1.5, 1.0]))
    assert e.value.code == fg.FBC_ERR_RANGE


def test_duplicate_edges_summed(fg):
    """DirectedWeightedGraph.h:154-165: a repeated pair has its weights summed."""
    g = fg.Graph.from_edges(np.array([0, 0, 1, 0, 2], np.int32), np.array([1, 2, 2, 1, 0], np.int32),
                            np.array([2.0, 5.0, 1.0, 2.0, 1.0]))
    rp, col, w = g.csr()
    assert g.n == 3 and g.m == 4
    assert list(col[rp[0]:rp[1]]) == [1, 2] and list(w[rp[0]:rp[1]]) == [4.0, 5.0]


def _clustered_inputs(fg):
    import os
    from conftest import GOLDEN

    z = np.load(os.path.join(GOLDEN, "grid256_clustered.npz"))
    off, cv, boff, bv = z["cluster_off"], z["cluster_vertices"], z["border_off"], z["borders"]
    poff, pv, kv = z["pivot_off"], z["pivots"], z["cards"]
    keep = [c for c in range(off.size - 1) if boff[c + 1] > boff[c]]
    cs = fg.ClusterSet.from_lists([cv[off[c]:off[c + 1]] for c in keep],
                                  [bv[boff[c]:boff[c + 1]] for c in keep])
    piv = [pv[poff[c]:poff[c + 1]] for c in keep]
    crd = [kv[poff[c]:poff[c + 1]] for c in keep]
    return z, keep, cs, piv, crd


@pytest.mark.parametrize("prec,sched", [(0, 0), (0, 1), (1, 1)])
def test_grid256_clustered_matches_reference(fg, prec, sched):
    """The full clustered pipeline (reference partition + pivots) against the reference's own
    ClusteredBrandeBC::computeBC output.  The result is a cancellation (intra + sum dep*card -
    sum intra*card, most entries negative), so the bound is |err| / max|BC|; intra BC is
    checked elementwise."""
    z, keep, cs, piv, crd = _clustered_inputs(fg)
    el = graphs.WORKLOADS["grid256"]()
    g = fg.Graph.from_edgelist(el)
    tol = TOL_FP64 if prec == 0 else TOL_FP32C
    ev = fg.cluster_eval_batch(g, cs, prec, sched)
    assert rel_err(ev.intra_bc, z["intra_bc"]) <= tol
    bc = fg.clustered_bc(g, cs, piv, crd, prec, sched, ev=ev)
    golden = z["bc"]
    assert np.max(np.abs(bc - golden)) / np.max(np.abs(golden)) <= tol


def test_grid256_cluster_border_vectors(fg):
    """VertexInfo (border length, count) of three reference clusters: bit-exact."""
    z, keep, cs, piv, crd = _clustered_inputs(fg)
    el = graphs.WORKLOADS["grid256"]()
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    ev = fg.cluster_eval_batch(g, cs, fg.FP32C, fg.BATCHED)
    for c in (0, 11, len(keep) - 1):
        vs = cs.vertices[cs.off[c]:cs.off[c + 1]]
        b = cs.borders[cs.boff[c]:cs.boff[c + 1]]
        _, bd, bs = oracle.cluster_eval(og, vs, b)
        for i in range(vs.size):
            L, Cn = ev.vertex_info(c, i)
            assert np.array_equal(L, bd[i]) and np.array_equal(Cn.astype(np.float64), bs[i])


@pytest.mark.parametrize("prec", [0, 1])
def test_cluster_plan_replays(fg, prec):
    """A prepared sweep (captured CUDA graphs) gives the reference's intra BC and bit-exact border
    vectors on every replay, whichever kernels it captures: the shared-memory kernel alone (the
    default for these communities), both kernels (communities on either side of warp_max_n), or
    the frontier kernel alone (four sources per block).  A community above 32K vertices keeps the
    plan uncaptured: it runs the general path with the same results."""
    z, keep, cs, piv, crd = _clustered_inputs(fg)
    g = fg.Graph.from_edgelist(graphs.WORKLOADS["grid256"]())
    tol = TOL_FP64 if prec == 0 else TOL_FP32C
    base = fg.cluster_eval_batch(g, cs, prec, fg.PLAIN)
    old = fg.get_option("warp_max_n")
    try:
        for wmax, launches in ((old, 1), (900, 2), (64, 1)):
            fg.set_option("warp_max_n", wmax)
            plan = fg.ClusterPlan(g, cs, prec)
            assert plan.captured
            for _ in range(3):
                st = fg.Stats()
                ev = plan.run(st)
                assert st.launches == launches and st.units == cs.vertices.size
                assert (st.block_units > 0) == (wmax < old) and (st.warp_units > 0) == (wmax > 64)
                assert rel_err(ev.intra_bc, z["intra_bc"]) <= tol
                assert np.array_equal(ev.border_dist, base.border_dist)
                assert np.array_equal(ev.border_sigma, base.border_sigma)
            plan.free()
    finally:
        fg.set_option("warp_max_n", old)
    whole = fg.ClusterSet.from_lists([np.arange(g.n, dtype=np.int32)]).with_borders(g)
    plan = fg.ClusterPlan(g, whole, prec)
    assert not plan.captured
    ev = plan.run()
    ref = fg.cluster_eval_batch(g, whole, prec, fg.BATCHED)
    assert rel_err(ev.intra_bc, ref.intra_bc) <= tol


@pytest.mark.parametrize("sched", [0, 1])
def test_grid256_sources_bit_exact_both_schedules(fg, sched):
    """Distances, path counts and predecessor counts from the plain block kernel and from the
    batched frontier kernel (64-bit (dist|stamp) words, packed sigma|counter)."""
    el = graphs.WORKLOADS["grid256"]()
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    fg.set_option("debug_sched", sched)
    try:
        for src in (3, 40000):
            check_source(fg, g, og, src)
    finally:
        fg.set_option("debug_sched", 0)


def test_rgg_sources_bit_exact_batched(fg):
    el = graphs.rgg_knn(20000, seed=13)
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    fg.set_option("debug_sched", 1)
    try:
        for src in (0, 19999):
            check_source(fg, g, og, src)
    finally:
        fg.set_option("debug_sched", 0)


def test_rgg_batch_smallest_graphs(fg):
    """The 48-graph batching workload: its four smallest graphs, exact BC against the oracle."""
    els = sorted(graphs.rgg_batch(48), key=lambda e: e.n)[:4]
    gs = [fg.Graph.from_edgelist(e) for e in els]
    for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
        for sched in (fg.PLAIN, fg.BATCHED):
            outs = fg.multi_exact_bc(gs, prec, sched)
            for e, o in zip(els, outs):
                assert rel_err(o, oracle.exact_bc(oracle.CSR.from_edgelist(e))) <= tol


def test_rgg_batch_all_graphs(fg):
    """The whole 48-graph batch (n from 1,128 to 58,453) in one persistent launch, as the batching
    bench runs it: the 24 smallest graphs' exact BC against the oracle's (FP64 1e-9, FP32C 1e-6),
    every graph's FP32C result within 1e-6 of its FP64 one, and on every one of the 48 graphs a
    seeded sample of 6 sources through the batched kernels against the oracle."""
    import os

    threads = os.cpu_count() or 1
    els = graphs.rgg_batch(48)
    gs = [fg.Graph.from_edgelist(e) for e in els]
    f64 = fg.multi_exact_bc(gs, fg.FP64, fg.BATCHED)
    f32 = fg.multi_exact_bc(gs, fg.FP32C, fg.BATCHED)
    by_size = sorted(range(len(els)), key=lambda i: els[i].n)
    for i in by_size[:24]:
        ref = oracle.exact_bc(oracle.CSR.from_edgelist(els[i]), threads=threads)
        assert rel_err(f64[i], ref) <= TOL_FP64, f"graph {i} (n={els[i].n})"
        assert rel_err(f32[i], ref) <= TOL_FP32C, f"graph {i} (n={els[i].n})"
    for i, e in enumerate(els):
        assert rel_err(f32[i], f64[i]) <= TOL_FP32C, f"graph {i} (n={e.n})"
        src = np.unique(graphs.rand_int(31, i, np.arange(6), 0, e.n - 1)).astype(np.int32)
        ref = oracle.exact_bc_sources(oracle.CSR.from_edgelist(e), src, threads=threads)
        got = fg.dependency_batch(gs[i], src, None, fg.FP64, fg.BATCHED)
        assert rel_err(got, ref) <= TOL_FP64, f"graph {i} (n={e.n})"


def test_grid512_precision_form(fg):
    """Precision configuration (512x512 grid): on 512 sampled sources the FP32-compensated form
    stays within 1e-6 of the FP64 form (itself within 1e-9 of the oracle on a subset), and
    distances and path counts are bit-exact."""
    el = graphs.WORKLOADS["grid512"]()
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    src = np.unique(graphs.rand_int(5, 1, np.arange(512), 0, el.n - 1)).astype(np.int32)
    f64 = fg.dependency_batch(g, src, None, fg.FP64, fg.BATCHED)
    f32 = fg.dependency_batch(g, src, None, fg.FP32C, fg.BATCHED)
    assert rel_err(f32, f64) <= TOL_FP32C
    ref = oracle.exact_bc_sources(og, src[:8], threads=8)
    got = fg.dependency_batch(g, src[:8], None, fg.FP64, fg.BATCHED)
    assert rel_err(got, ref) <= TOL_FP64
    fg.set_option("debug_sched", 1)
    try:
        check_source(fg, g, og, int(src[0]))
    finally:
        fg.set_option("debug_sched", 0)


def test_grid2048_full_size_sources(fg):
    """Full form graph (4,194,304 vertices): two sources bit-exact against the oracle through both
    block kernels, and FP32C vs FP64 on 32 sampled sources."""
    el = graphs.WORKLOADS["grid2048"]()
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    for sched, s in ((0, 1234567), (1, el.n - 1)):
        fg.set_option("debug_sched", sched)
        try:
            dist, sig, dlt, npred = fg.sssp_debug(g, s)
        finally:
            fg.set_option("debug_sched", 0)
        od, osg, odl, order, preds = oracle.sssp_dump(og, s)
        assert np.array_equal(np.where(dist < 0, np.inf, dist.astype(np.float64)), od)
        assert np.array_equal(sig.astype(np.float64), osg)
        assert np.array_equal(npred, np.array([len(p) for p in preds]))
        assert rel_err(dlt[od < np.inf], odl[od < np.inf]) <= TOL_FP64
    src = np.arange(7, el.n, el.n // 32, dtype=np.int32)[:32]
    f64 = fg.dependency_batch(g, src, None, fg.FP64, fg.BATCHED)
    f32 = fg.dependency_batch(g, src, None, fg.FP32C, fg.BATCHED)
    assert rel_err(f32, f64) <= TOL_FP32C


def test_large_path_counts_are_recomputed_exactly(fg):
    """Random geometric graphs with small tied weights have path counts above 2^48 (the batched
    block kernel's packed field): those units are recomputed by the plain kernel, results equal
    the FP64 plain path and the oracle."""
    el = graphs.rgg_knn(51013, seed=7, gid=23)  # the batch's second largest graph
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    src = np.arange(0, el.n, el.n // 64, dtype=np.int32)[:64]
    _, sig, _, _ = fg.sssp_debug(g, int(src[0]))
    a = fg.dependency_batch(g, src, None, fg.FP64, fg.BATCHED)
    b = fg.dependency_batch(g, src, None, fg.FP64, fg.PLAIN)
    assert rel_err(a, b) <= TOL_FP64
    assert rel_err(a, oracle.exact_bc_sources(og, src, threads=8)) <= TOL_FP64


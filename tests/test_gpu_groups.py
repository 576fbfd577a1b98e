"""The frontier kernel with K sources per block (option "group"): the K sources of a block share
rounds and levels and interleave their per-vertex state; results must not depend on K.  Groups
are padded when a segment's source count is not a multiple of K; a group whose path counts or
queues outgrow the kernel hands every source of the group to the plain kernel."""
import numpy as np
import pytest

import graphs
import oracle
from test_gpu_parity import TOL_FP32C, TOL_FP64, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture
def group(fg, request):
    old = fg.get_option("group")
    fg.set_option("group", request.param)
    yield request.param
    fg.set_option("group", old)


@pytest.mark.parametrize("group", [1, 2, 4], indirect=True)
@pytest.mark.parametrize("prec", [0, 1])
def test_pivot_batch_grouped(fg, group, prec):
    el = graphs.WORKLOADS["grid256"]()
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    rng = np.random.default_rng(5)
    piv = rng.choice(el.n, 23, replace=False).astype(np.int32)  # not a multiple of 2 or 4
    cards = rng.integers(1, 9, piv.size).astype(np.float64)
    st = fg.Stats()
    got = fg.dependency_batch(g, piv, cards, prec, fg.BATCHED, stats=st)
    assert st.group == group
    assert rel_err(got, oracle.pivot_batch(og, piv, cards)) <= (TOL_FP64 if prec == 0 else TOL_FP32C)


@pytest.mark.parametrize("group", [2, 4], indirect=True)
def test_cluster_eval_grouped_frontier(fg, group):
    """Clusters pushed to the frontier kernel (warp_max_n below every cluster size): intra BC and
    bit-exact border vectors for every source of every group."""
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
    old = fg.get_option("warp_max_n")
    fg.set_option("warp_max_n", 16)
    try:
        for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
            st = fg.Stats()
            ev = fg.cluster_eval_batch(g, cs, prec, fg.BATCHED, stats=st)
            assert st.group == group and st.warp_units == 0
            assert rel_err(ev.intra_bc, ref_bc) <= tol
            for c, (bd, bs) in enumerate(refs):
                for i in range(len(clusters[c])):
                    L, Cn = ev.vertex_info(c, i)
                    assert np.array_equal(L, bd[i]) and np.array_equal(Cn.astype(np.float64), bs[i])
    finally:
        fg.set_option("warp_max_n", old)


@pytest.mark.parametrize("group", [4], indirect=True)
def test_grouped_debug_and_retry(fg, group):
    """Path counts above 2^48 inside a group of four: the whole group is recomputed by the plain
    kernel with 64-bit counts; the per-source dump of a grouped run is bit-exact."""
    el = graphs.rgg_knn(51013, seed=7, gid=23)
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    src = np.arange(0, el.n, el.n // 64, dtype=np.int32)[:61]
    a = fg.dependency_batch(g, src, None, fg.FP64, fg.BATCHED)
    assert rel_err(a, oracle.exact_bc_sources(og, src, threads=8)) <= TOL_FP64
    fg.set_option("debug_sched", 1)
    try:
        from test_gpu_parity import check_source
        check_source(fg, g, og, 777)
    finally:
        fg.set_option("debug_sched", 0)


@pytest.mark.parametrize("group", [4], indirect=True)
def test_grid2048_grouped_matches_oracle(fg, group):
    """4,194,304-vertex grid, wide blocks: 8 sources four per block and one per block, FP64 within
    1e-9 and FP32C within 1e-6 of the oracle."""
    import os

    el = graphs.WORKLOADS["grid2048"]()
    g = fg.Graph.from_edgelist(el)
    src = np.arange(101, el.n, el.n // 8, dtype=np.int32)[:8]
    ref = oracle.exact_bc_sources(oracle.CSR.from_edgelist(el), src, threads=os.cpu_count() or 1)
    st = fg.Stats()
    a = fg.dependency_batch(g, src, None, fg.FP64, fg.BATCHED, stats=st)
    assert st.group == 4
    b = fg.dependency_batch(g, src, None, fg.FP32C, fg.BATCHED)
    fg.set_option("group", 1)
    c = fg.dependency_batch(g, src, None, fg.FP64, fg.BATCHED)
    assert rel_err(a, ref) <= TOL_FP64
    assert rel_err(c, ref) <= TOL_FP64
    assert rel_err(b, ref) <= TOL_FP32C


def test_mixed_segment_sizes_split_launches(fg):
    """A batch with graphs on both sides of the 32K-vertex line runs as two frontier launches
    (grouped small segments, then one source per block): every graph's exact BC equals its
    single-graph run."""
    els = [graphs.rgg_knn(n, seed=17, gid=i) for i, n in enumerate([6000, 33000, 9000])]
    gs = [fg.Graph.from_edgelist(e) for e in els]
    old = fg.get_option("warp_max_n")
    fg.set_option("warp_max_n", 0)  # every graph on the frontier kernel
    try:
        outs = fg.multi_exact_bc(gs, fg.FP64, fg.BATCHED)
        for gr, o in zip(gs, outs):
            assert rel_err(o, fg.exact_bc(gr, fg.FP64, fg.BATCHED)) <= TOL_FP64
    finally:
        fg.set_option("warp_max_n", old)


def _hub_graph(n=2500, hub_in=300, seed=3):
    """A ring with random weights plus one vertex with `hub_in` in-edges (forces the 16-bit
    counter layout of the frontier kernel)."""
    rng = np.random.default_rng(seed)
    src = list(range(n)) + list(range(1, n))
    dst = [(i + 1) % n for i in range(n)] + [i - 1 for i in range(1, n)]
    feeders = rng.choice(np.arange(1, n), hub_in, replace=False)
    src += list(feeders)
    dst += [0] * hub_in
    src += [0] * 5
    dst += list(rng.choice(np.arange(1, n), 5, replace=False))
    w = rng.integers(1, 50, len(src)).astype(np.float64)
    return np.array(src, np.int32), np.array(dst, np.int32), w


@pytest.mark.parametrize("kind", ["hub", "dense_rows"])
def test_counter_layouts(fg, kind):
    """8-bit counters and masks (rows of 8+ edges re-tested) on a graph with long rows, 16-bit ones
    on a graph with a 300-in-edge vertex: both equal the oracle."""
    if kind == "hub":
        s, d, w = _hub_graph()
        g = fg.Graph.from_edges(s, d, w)
        og = oracle.CSR(*g.csr())
    else:
        el = graphs.rgg_knn(3000, k=12, seed=21)
        g = fg.Graph.from_edgelist(el)
        og = oracle.CSR.from_edgelist(el)
    src = np.arange(0, g.n, max(1, g.n // 40), dtype=np.int32)[:40]
    ref = oracle.exact_bc_sources(og, src, threads=8)
    old = fg.get_option("warp_max_n")
    fg.set_option("warp_max_n", 0)  # the frontier kernel, not the shared-memory one
    try:
        for prec, tol in ((fg.FP64, TOL_FP64), (fg.FP32C, TOL_FP32C)):
            got = fg.dependency_batch(g, src, None, prec, fg.BATCHED)
            assert rel_err(got, ref) <= tol
    finally:
        fg.set_option("warp_max_n", old)

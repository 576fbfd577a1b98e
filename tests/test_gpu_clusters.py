"""Cluster subgraphs built on the device (border discovery, local CSR extraction): borders
equal SubGraph's definition (SubGraph.h:59-148: an end of an edge between different clusters,
listed in ascending id) for shuffled cluster lists too, and bad cluster lists are rejected with
FBC_ERR_INVALID_ARG before any kernel reads them."""
import numpy as np
import pytest

import graphs
import oracle
from test_gpu_parity import TOL_FP64, rel_err

pytestmark = pytest.mark.gpu


def _host_borders(el, clusters):
    cid = np.full(el.n, -1, np.int64)
    for c, vs in enumerate(clusters):
        cid[vs] = c
    cross = cid[el.src] != cid[el.dst]
    isb = np.zeros(el.n, bool)
    isb[el.src[cross]] = True
    isb[el.dst[cross]] = True
    return [np.sort(vs[isb[vs]]) for vs in clusters]


def _tiles(el, side, tile, rng=None):
    ids = np.arange(el.n)
    t = (ids // side) // tile * (side // tile) + (ids % side) // tile
    out = [ids[t == k].astype(np.int32) for k in range((side // tile) ** 2)]
    if rng is not None:
        out = [rng.permutation(vs).astype(np.int32) for vs in out]
    return out


@pytest.mark.parametrize("shuffled", [False, True])
def test_device_borders_match_subgraph_rule(fg, shuffled):
    el = graphs.road_grid(64, 64, seed=9)
    g = fg.Graph.from_edgelist(el)
    clusters = _tiles(el, 64, 16, np.random.default_rng(1) if shuffled else None)
    cs = fg.ClusterSet.from_lists(clusters).with_borders(g)
    want = _host_borders(el, clusters)
    for c in range(len(clusters)):
        assert np.array_equal(cs.borders[cs.boff[c]:cs.boff[c + 1]], want[c])


def test_shuffled_clusters_evaluate_like_sorted(fg):
    """Vertex order inside a cluster changes local ids, not results: intra BC and per-vertex
    border vectors equal the oracle's."""
    el = graphs.road_grid(64, 64, seed=9)
    og = oracle.CSR.from_edgelist(el)
    g = fg.Graph.from_edgelist(el)
    clusters = _tiles(el, 64, 16, np.random.default_rng(2))
    cs = fg.ClusterSet.from_lists(clusters).with_borders(g)
    ref_bc = np.zeros(el.n)
    for sched in (fg.PLAIN, fg.BATCHED):
        ev = fg.cluster_eval_batch(g, cs, fg.FP64, sched)
        ref_bc[:] = 0
        for c, vs in enumerate(clusters):
            b = cs.borders[cs.boff[c]:cs.boff[c + 1]]
            _, bd, bs = oracle.cluster_eval(og, vs, b, ref_bc)
            for i in range(0, vs.size, 37):
                L, Cn = ev.vertex_info(c, i)
                assert np.array_equal(L, bd[i]) and np.array_equal(Cn.astype(np.float64), bs[i])
        assert rel_err(ev.intra_bc, ref_bc) <= TOL_FP64


def test_bad_cluster_lists_rejected(fg):
    el = graphs.road_grid(32, 32, seed=3)
    g = fg.Graph.from_edgelist(el)
    good = _tiles(el, 32, 16)
    dup = [good[0], np.concatenate([good[1], good[0][:1]]).astype(np.int32)]
    out_of_range = [good[0], np.array([el.n + 5], np.int32)]
    for bad in (dup, out_of_range):
        with pytest.raises(fg.FbcError) as e:
            fg.cluster_eval_batch(g, fg.ClusterSet.from_lists(bad), fg.FP64, fg.BATCHED)
        assert e.value.code == fg.FBC_ERR_INVALID_ARG
    wrong_border = fg.ClusterSet.from_lists(good[:2], [good[1][:3], good[0][:3]])
    with pytest.raises(fg.FbcError) as e:
        fg.cluster_eval_batch(g, wrong_border, fg.FP64, fg.BATCHED)
    assert e.value.code == fg.FBC_ERR_INVALID_ARG
    # the library stays usable
    ev = fg.cluster_eval_batch(g, fg.ClusterSet.from_lists(good), fg.FP64, fg.BATCHED)
    assert np.all(np.isfinite(ev.intra_bc))


def test_failed_plan_create_frees_its_buffers(fg):
    """A cluster plan whose creation is rejected half way (a border that is not one, found by the
    device border map after the plan's subgraph buffers exist) leaves no device memory behind,
    and a valid plan afterwards gives the batched sweep's values."""
    torch = pytest.importorskip("torch")
    el = graphs.road_grid(512, 512, seed=4)
    g = fg.Graph.from_edgelist(el)
    good = _tiles(el, 512, 128)
    wrong = fg.ClusterSet.from_lists(good[:2], [good[1][:3], good[0][:3]])
    with pytest.raises(fg.FbcError):
        fg.ClusterPlan(g, wrong, fg.FP64)  # first call: the library's own workspaces grow
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(20):
        with pytest.raises(fg.FbcError) as e:
            fg.ClusterPlan(g, wrong, fg.FP64)
        assert e.value.code == fg.FBC_ERR_INVALID_ARG
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    # each leaked attempt would hold the 512x512 cluster CSRs (about 9 MB)
    assert free0 - free1 < 32 << 20
    cs = fg.ClusterSet.from_lists(good[:4])
    plan = fg.ClusterPlan(g, cs, fg.FP64)
    got = plan.run()
    ref = fg.cluster_eval_batch(g, cs, fg.FP64, fg.BATCHED)
    plan.free()
    assert rel_err(got.intra_bc, ref.intra_bc) <= TOL_FP64
    assert np.array_equal(got.border_dist, ref.border_dist)
    assert np.array_equal(got.border_sigma, ref.border_sigma)

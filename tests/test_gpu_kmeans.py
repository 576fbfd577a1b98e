"""The k-means step of the clustered pivot selection on the device (fbc_kmeans) against the
reference's own selection: the 256x256 grid's Louvain communities (every one with borders; the
reference's KMeansPivotSelector output is in grid256_clustered.npz) and a community of the
2048x2048 grid (the reference's selection in grid2048_pivots.npz), from the engine's own border
vectors and exact classes -- pivots and weights equal, in the reference's order.  A set of the
oracle's restatement with random inputs checks the rounding and tie rules beyond those."""
import os

import numpy as np
import pytest

import graphs
import oracle
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _sets(fg, g, cs, bc, ev):
    """Exact classes (device) and their pivots' normalized border vectors, per cluster."""
    classes = fg.cluster_classes(g, cs, bc, ev)
    cp, sets = [], []
    for c, (piv, crd) in enumerate(classes):
        vs = cs.vertices[cs.off[c]:cs.off[c + 1]]
        pos = {int(v): i for i, v in enumerate(vs)}
        rows = np.array([pos[int(v)] for v in piv])
        nb = int(cs.boff[c + 1] - cs.boff[c])
        e0 = int(ev.entry_off[c])
        L = ev.border_dist[e0:e0 + vs.size * nb].reshape(vs.size, nb)[rows]
        Cn = ev.border_sigma[e0:e0 + vs.size * nb].reshape(vs.size, nb)[rows]
        L = L - L.min(axis=1, keepdims=True)  # VertexInfo::normalize
        cp.append(piv)
        sets.append((L, Cn.astype(np.int64).astype(np.int32), crd))
    return cp, sets


def test_kmeans_matches_reference_on_grid256(fg):
    z = np.load(os.path.join(GOLDEN, "grid256_clustered.npz"))
    g = fg.Graph.from_edgelist(graphs.WORKLOADS["grid256"]())
    keep = [c for c in range(z["cluster_off"].size - 1) if z["border_off"][c + 1] > z["border_off"][c]]
    cs = fg.ClusterSet.from_lists([z["cluster_vertices"][z["cluster_off"][c]:z["cluster_off"][c + 1]] for c in keep],
                                  [z["borders"][z["border_off"][c]:z["border_off"][c + 1]] for c in keep])
    ev = fg.cluster_eval_batch(g, cs, fg.FP64, fg.BATCHED)
    zc = np.load(os.path.join(GOLDEN, "grid256_classes.npz"))
    cp, sets = _sets(fg, g, cs, zc["intra_bc"], ev)  # the BC the reference's selector compared
    for k, c in enumerate(keep):  # the exact classes are the reference's
        assert np.array_equal(cp[k], zc["pivots"][zc["class_off"][c]:zc["class_off"][c + 1]])
    got = fg.kmeans_pivot_sets(cp, sets)
    for k, c in enumerate(keep):
        p0, p1 = z["pivot_off"][c], z["pivot_off"][c + 1]
        assert np.array_equal(got[k][0], z["pivots"][p0:p1]), f"community {c}"
        assert np.array_equal(got[k][1], z["cards"][p0:p1]), f"community {c}"


def test_kmeans_matches_reference_on_grid2048_community(fg):
    cid = np.load(os.path.join(GOLDEN, "grid2048_partition.npz"))["community"].astype(np.int64)
    pz = np.load(os.path.join(GOLDEN, "grid2048_pivots.npz"))
    c = int(pz["clusters"][0])
    g = fg.Graph.from_edgelist(graphs.WORKLOADS["grid2048"]())
    cs = fg.ClusterSet.from_lists([np.nonzero(cid == c)[0].astype(np.int32)]).with_borders(g)
    ev = fg.cluster_eval_batch(g, cs, fg.FP64, fg.BATCHED)
    cp, sets = _sets(fg, g, cs, ev.intra_bc, ev)
    (piv, w), = fg.kmeans_pivot_sets(cp, sets)
    assert np.array_equal(piv, pz["pivots"][pz["pivot_off"][0]:pz["pivot_off"][1]])
    assert np.array_equal(w, pz["cards"][pz["pivot_off"][0]:pz["pivot_off"][1]])


def test_kmeans_matches_oracle_on_random_sets(fg):
    """Random small sets with many equal distances (few distinct values): the device and the
    oracle's restatement agree on every centroid and weight, duplicates included."""
    rng = np.random.default_rng(3)
    sets = []
    for s in range(12):
        npv, nb = int(rng.integers(3, 300)), int(rng.integers(0, 12))
        L = rng.integers(0, 4, (npv, nb)).astype(np.float64)
        L -= L.min(axis=1, keepdims=True) if nb else 0
        sets.append((L, rng.integers(0, 3, (npv, nb)).astype(np.int32), rng.integers(1, 9, npv).astype(np.int32)))
    got = fg.kmeans(sets)
    for (L, Cn, w), (idx, gw) in zip(sets, got):
        oi, ow = oracle.kmeans_pivots(L, Cn, w)
        # the oracle removes duplicates: compare after the same removal
        seen, di, dw = set(), [], []
        for i, x in zip(idx.tolist(), gw.tolist()):
            if i not in seen:
                seen.add(i)
                di.append(i)
                dw.append(x)
        assert di == oi.tolist() and dw == ow.tolist()

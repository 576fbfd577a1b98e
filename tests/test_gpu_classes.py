"""Topological classes on the device (VertexInfoPivotSelector::selectPivots for every cluster)
against the reference's own selector on the 256x256 grid's Louvain partition
(tests/golden/grid256_classes.npz, made by the reference harness): given the reference's
intra-cluster BC, the classes, their order, pivots and cardinalities are identical."""
import os

import numpy as np
import pytest

import graphs
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_classes_match_reference_selector(fg):
    z = np.load(os.path.join(GOLDEN, "grid256_clustered.npz"))
    k = np.load(os.path.join(GOLDEN, "grid256_classes.npz"))
    off, cv = z["cluster_off"], z["cluster_vertices"]
    g = fg.Graph.from_edgelist(graphs.WORKLOADS["grid256"]())
    cs = fg.ClusterSet.from_lists([cv[off[c]:off[c + 1]] for c in range(off.size - 1)]).with_borders(g)
    ev = fg.cluster_eval_batch(g, cs, fg.FP64, fg.BATCHED)
    got = fg.cluster_classes(g, cs, k["intra_bc"], ev)
    coff = k["class_off"]
    for c in range(off.size - 1):
        p, n = got[c]
        assert np.array_equal(p, k["pivots"][coff[c]:coff[c + 1]]), f"cluster {c}"
        assert np.array_equal(n, k["cards"][coff[c]:coff[c + 1]]), f"cluster {c}"
    assert sum(n.sum() for _, n in got) == sum(np.diff(off)[c] for c in range(off.size - 1) if cs.boff[c + 1] > cs.boff[c])


def test_classes_tiny_cluster_known_answer(fg):
    """Two clusters of a path 0-1-2-3 | 4-5: hand-checked classes."""
    src = np.array([0, 1, 1, 2, 2, 3, 3, 4, 4, 5], np.int32)
    dst = np.array([1, 0, 2, 1, 3, 2, 4, 3, 5, 4], np.int32)
    w = np.ones(src.size)
    g = fg.Graph.from_edges(src, dst, w)
    cs = fg.ClusterSet.from_lists([np.array([0, 1, 2, 3], np.int32), np.array([4, 5], np.int32)]).with_borders(g)
    ev = fg.cluster_eval_batch(g, cs, fg.FP64, fg.BATCHED)
    bc = np.array([0.0, 2.0, 2.0, 0.0, 0.0, 0.0])
    got = fg.cluster_classes(g, cs, bc, ev)
    # cluster 0 (border 3): vectors to the border (length - min, count): all (0, 1) -> one class
    # of 4; non-borders 0, 1, 2 with bc 0, 2, 2 -> pivot 0
    assert list(got[0][0]) == [0] and list(got[0][1]) == [4]
    # cluster 1 (border 4): one class of 2, its only non-border member 5 is the pivot
    assert list(got[1][0]) == [5] and list(got[1][1]) == [2]

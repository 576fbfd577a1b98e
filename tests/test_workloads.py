"""The seeded workload generators are reproducible: the golden fixtures (the reference's runs on
these graphs) and the bench configurations depend on them edge for edge (CPU only)."""
import hashlib

import numpy as np
import pytest

import graphs


def _digest(el):
    h = hashlib.sha256()
    for a in (el.src, el.dst, el.w):
        h.update(np.ascontiguousarray(a, np.int64).tobytes())
    return h.hexdigest()[:16]


@pytest.mark.parametrize("name,n,m,digest", [
    ("grid32", 1024, 3968, "ac21d0068a03fda3"),
    ("grid256", 65536, 248528, "513ac0956aea3b3c"),
    ("grid512", 262144, 995164, "9d895bd3c3a0e9b3"),
    ("grid2048", 4194304, 15937326, "3e54ba2f8bfe20f6"),  # the partition golden's graph (~10 s)
])
def test_road_grids(name, n, m, digest):
    el = graphs.WORKLOADS[name]()
    assert (el.n, el.m, _digest(el)) == (n, m, digest)


def test_random_geometric_graph():
    el = graphs.rgg_knn(1500, seed=11)
    assert (el.n, el.m, _digest(el)) == (1500, 5576, "e9cee4f4855e2191")


def test_batch_sizes():
    sz = graphs.rgg_sizes()
    assert len(sz) == 48 and 1024 <= min(sz) and max(sz) <= 65536

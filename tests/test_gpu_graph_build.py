"""Edge list -> CSR on the device (DirectedWeightedGraph.h:67-96, 136-170 rules): the device build
gives exactly the host build's CSR (rows ascending, repeated pairs summed in input order) for
shuffled input with duplicates, falls back to the host for rows longer than the device sort
handles, and rejects the same inputs with the same status codes."""
import numpy as np
import pytest

import graphs

pytestmark = pytest.mark.gpu


@pytest.fixture
def device_min(fg):
    old = fg.get_option("csr_device_min_m")
    yield lambda v: fg.set_option("csr_device_min_m", v)
    fg.set_option("csr_device_min_m", old)


def _both(fg, device_min, src, dst, w):
    out = []
    for v in (1 << 40, 0):  # host build, device build
        device_min(v)
        g = fg.Graph.from_edges(src, dst, w)
        out.append(g.csr())
        g.free()
    return out


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_device_build_matches_host(fg, device_min):
    el = graphs.WORKLOADS["grid256"]()
    rng = np.random.default_rng(4)
    # shuffled, with 5% of the edges repeated (weights then summed)
    rep = rng.choice(el.m, el.m // 20, replace=False)
    src = np.concatenate([el.src, el.src[rep]])
    dst = np.concatenate([el.dst, el.dst[rep]])
    w = np.concatenate([el.w, el.w[rep]]).astype(np.float64)
    p = rng.permutation(src.size)
    h, d = _both(fg, device_min, src[p].astype(np.int32), dst[p].astype(np.int32), w[p])
    assert _same(h, d)
    rp, col, ww = d
    assert rp[-1] == el.m


def test_device_build_half_weights_sum_to_integers(fg, device_min):
    src = np.array([0, 1, 0, 2, 0], np.int32)
    dst = np.array([1, 2, 1, 0, 2], np.int32)
    w = np.array([0.5, 3.0, 0.5, 1.0, 2.0])
    h, d = _both(fg, device_min, src, dst, w)
    assert _same(h, d)
    assert list(d[1][d[0][0]:d[0][1]]) == [1, 2] and list(d[2][d[0][0]:d[0][1]]) == [1.0, 2.0]


def test_long_rows_fall_back_to_host(fg, device_min):
    n = 3000
    src = np.concatenate([np.zeros(n - 1, np.int32), np.arange(1, n, dtype=np.int32)])
    dst = np.concatenate([np.arange(1, n, dtype=np.int32), np.zeros(n - 1, np.int32)])
    w = np.ones(src.size)
    h, d = _both(fg, device_min, src, dst, w)
    assert _same(h, d)


def test_device_build_rejects_like_host(fg, device_min):
    cases = [
        (np.array([0, 1], np.int32), np.array([1, 5], np.int32), np.array([1.0, 1.0]), fg.FBC_ERR_INVALID_ARG),
        (np.array([0, 1], np.int32), np.array([1, 0], np.int32), np.array([1.0, 0.0]), fg.FBC_ERR_INVALID_ARG),
        (np.array([0, 1], np.int32), np.array([1, 0], np.int32), np.array([1.5, 1.0]), fg.FBC_ERR_RANGE),
        (np.array([0, -1], np.int32), np.array([1, 0], np.int32), np.array([1.0, 1.0]), fg.FBC_ERR_INVALID_ARG),
    ]
    for src, dst, w, code in cases:
        for v in (1 << 40, 0):
            device_min(v)
            with pytest.raises(fg.FbcError) as e:
                fg.Graph.from_edges(src, dst, w)
            assert e.value.code == code

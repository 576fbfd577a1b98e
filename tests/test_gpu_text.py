"""Edge-list text parsed on the device (fbc_graph_from_text): the graph the reference's parser
builds from the same bytes (tests/golden/text, made by DirectedWeightedGraph(std::istream&)), the
text oracle's reading of seeded texts with random layout and number forms, weights converted on
the host (long significands), long rows built on the host, and the same rejections."""
import numpy as np
import pytest

import graphs
import text_cases
import text_oracle as to

pytestmark = pytest.mark.gpu


def _csr(fg, text):
    g = fg.Graph.from_text(text)
    try:
        return g.csr()
    finally:
        g.free()


def _same(a, b):
    return all(np.array_equal(np.asarray(x), np.asarray(y)) for x, y in zip(a, b))


@pytest.mark.parametrize("name", text_cases.cases())
def test_reference_fixtures(fg, name):
    text, want = text_cases.load(name)
    if isinstance(want, str):
        with pytest.raises(fg.FbcError) as e:
            fg.Graph.from_text(text)
        assert e.value.code == fg.FBC_ERR_INVALID_ARG and want in str(e.value)
        return
    assert _same(_csr(fg, text), want)


def _random_text(rng, n, m, slow_share=0.0):
    src = rng.integers(0, n, m)
    src[:n] = np.arange(n)
    dst = rng.integers(0, n, m)
    w = rng.integers(1, 1000, m)
    seps = np.array([b" ", b"\t", b"   ", b" \t"], object)
    ends = np.array([b"\n", b"\r\n", b"\n\n", b"\t\n"], object)
    sp = seps[rng.integers(0, 4, m)]
    en = ends[rng.integers(0, 4, m)]
    slow = rng.random(m) < slow_share
    parts = []
    for i in range(m):
        x = int(w[i])
        ws = (b"%d.0000000000000000000000001" % x) if slow[i] else (b"%d" % x if i % 3 else b"%de-2" % (100 * x))
        parts.append(b"%d%s%d%s%s%s" % (src[i], sp[i], dst[i], sp[i], ws, en[i]))
    return b"".join(parts)


@pytest.mark.parametrize("slow_share", [0.0, 0.3])
def test_random_texts_match_oracle(fg, slow_share):
    rng = np.random.default_rng(5)
    text = _random_text(rng, 20000, 120000, slow_share)
    want = to.csr_from_edges(*to.parse_edge_text(text))
    assert _same(_csr(fg, text), want)


def test_road_grid_text_matches_edge_list(fg):
    el = graphs.WORKLOADS["grid512"]()
    lines = np.char.add(np.char.add(np.char.add(el.src.astype("S"), b" "),
                                    np.char.add(el.dst.astype("S"), b" ")),
                        np.char.add(el.w.astype(np.int64).astype("S"), b"\n"))
    text = b"".join(lines.tolist())
    g = fg.Graph.from_edgelist(el)
    want = g.csr()
    g.free()
    assert _same(_csr(fg, text), want)


def test_long_rows_built_on_the_host(fg):
    n = 3000
    rows = [b"0 %d 1\n" % v for v in range(1, n)] + [b"%d 0 2\n" % v for v in range(1, n)]
    text = b"".join(rows)
    assert _same(_csr(fg, text), to.csr_from_edges(*to.parse_edge_text(text)))


def test_empty_and_blank_texts(fg):
    for text in (b"", b" \n\t\r\n  "):
        g = fg.Graph.from_text(text)
        assert (g.n, g.m) == (0, 0)
        for sched in (fg.PLAIN, fg.BATCHED):
            assert fg.exact_bc(g, fg.FP64, sched).size == 0
        g.free()


@pytest.mark.parametrize("text,words", [
    (b"0 1 2\n1 0", "ends inside an edge"),
    (b"0 1 2\n1.5 0 3\n", "edge 1: a vertex id"),
    (b"0 99999999999 2\n", "edge 0: a vertex id"),
    (b"0 1 2\n1 0 2x\n", "greater than zero (edge 1)"),
    (b"0 1 2\n1 0 -0.0\n", "greater than zero (edge 1)"),
    (b"0 1 2\n1 0 +\n", "greater than zero (edge 1)"),
    (b"0 1 1e-400\n", "greater than zero (edge 0)"),
    (b"0 1 2\n1 0 2.5\n", "integers below 2^31"),
])
def test_rejections(fg, text, words):
    with pytest.raises(fg.FbcError) as e:
        fg.Graph.from_text(text)
    assert words in str(e.value)


def test_reading_ends_at_an_overflowing_weight(fg):
    # errors after the end of reading are never seen, as in the reference's loop
    text = b"0 1 2\n1 0 3\n1 0 1e400\n1.5 q 0\n7"
    rp, col, w = _csr(fg, text)
    assert list(rp) == [0, 1, 2] and list(col) == [1, 0] and list(w) == [2.0, 3.0]
    # a host-converted weight of a long significand still ends the reading when it overflows
    text = b"0 1 2\n1 0 3\n1 0 " + b"9" * 400 + b"\n1 1 0\n"
    rp, col, w = _csr(fg, text)
    assert list(col) == [1, 0]


def test_from_file(fg, tmp_path):
    text, want = text_cases.load("mixed")
    p = tmp_path / "g.txt"
    p.write_bytes(text)
    g = fg.Graph.from_file(str(p))
    assert _same(g.csr(), want)
    g.free()


def test_many_host_converted_weights(fg):
    # every weight past the device conversion (26 significant digits): the host converts them on
    # several threads; an overflowing one late in the text still ends the reading there
    rng = np.random.default_rng(8)
    n, m = 5000, 150000
    src = rng.integers(0, n, m)
    src[:n] = np.arange(n)
    dst = rng.integers(0, n, m)
    w = rng.integers(1, 100, m)
    lines = [b"%d %d %d.0000000000000000000000001\n" % (a, b, c) for a, b, c in zip(src, dst, w)]
    text = b"".join(lines)
    want = to.csr_from_edges_c(*to.parse_edge_text_c(text))
    assert _same(_csr(fg, text), want)
    cut = 140000
    text2 = b"".join(lines[:cut] + [b"0 1 1" + b"0" * 400 + b"\n"] + lines[cut:])
    want2 = to.csr_from_edges_c(*to.parse_edge_text_c(text2))
    got2 = _csr(fg, text2)
    assert _same(got2, want2) and int(got2[0][-1]) <= cut


def test_dwg_text_constructor_getters(fg):
    """DirectedWeightedGraph.cpp:11-40 (the reference's graph test) on DWGtext.txt parsed on the
    device: 9 vertices, 16 edges, the forward and backward stars of vertex 4, edge weights."""
    import os

    from conftest import GOLDEN

    g = fg.Graph.from_file(os.path.join(GOLDEN, "DWGtext.txt"))
    assert (g.n, g.m) == (9, 16)
    rp, col, w = g.csr()
    g.free()
    fs = dict(zip(col[rp[4]:rp[5]].tolist(), w[rp[4]:rp[5]].tolist()))
    assert fs == {5: 1.0, 6: 5.0, 8: 3.0}
    src = np.repeat(np.arange(9), np.diff(rp))
    bs = {int(s): float(x) for s, d, x in zip(src, col, w) if d == 4}
    assert bs == {0: 7.0, 2: 4.0, 3: 3.0}

    def edge(a, b):
        row = dict(zip(col[rp[a]:rp[a + 1]].tolist(), w[rp[a]:rp[a + 1]].tolist()))
        return row.get(b, 0.0)

    assert edge(7, 5) == 2 and edge(0, 1) == 4 and edge(1, 0) == 0


def test_long_ids_and_space_runs(fg):
    # 7- and 8-digit ids (the eight-byte fast path takes tokens of at most 8 bytes with a space
    # in view) and runs of 1..12 spaces or tabs between tokens, against the oracle
    rng = np.random.default_rng(12)
    n, m = 12_000_000, 60000
    src = rng.integers(0, n, m)
    dst = rng.integers(0, n, m)
    src[0] = n - 1
    w = rng.integers(1, 150, m)
    seps = [b" " * k for k in range(1, 13)] + [b"\t" * k for k in (1, 7, 8, 9)]
    parts = []
    for i in range(m):
        a = seps[rng.integers(len(seps))]
        b = seps[rng.integers(len(seps))]
        parts.append(b"%d%s%d%s%d\n" % (src[i], a, dst[i], b, w[i]))
    text = b"".join(parts)
    want = to.csr_from_edges_c(*to.parse_edge_text_c(text))
    assert _same(_csr(fg, text), want)

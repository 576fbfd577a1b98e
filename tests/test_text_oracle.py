"""The edge-list text oracle pinned to the reference's own parser (DirectedWeightedGraph(std::
istream&), DirectedWeightedGraph.h:67-96) on the fixtures of tests/golden/text (CPU only)."""
import numpy as np
import pytest

import text_cases
import text_oracle as to


@pytest.mark.parametrize("name", text_cases.cases())
def test_oracle_reads_like_the_reference(name):
    text, want = text_cases.load(name)
    if isinstance(want, str):
        assert want == "Edge weight must be greater than zero"
        with pytest.raises(to.TextError) as e:
            to.parse_edge_text(text)
        assert e.value.kind == "weight"
        return
    rp, col, w = to.csr_from_edges(*to.parse_edge_text(text))
    assert np.array_equal(rp, want[0]) and np.array_equal(col, want[1])
    assert np.array_equal(w, want[2])  # exact: both sides are correctly rounded


def test_oracle_undefined_cases_are_errors():
    for text, kind, edge in [(b"0 1 2\n1 0", "incomplete", 1), (b"0 1 2\n1.5 0 3\n", "id", 1),
                             (b"0 99999999999 2\n", "id", 0), (b"0 1 2x\n", "weight", 0),
                             (b"0 1 2\n1 0 1e400\nx y z w\n", None, None)]:
        if kind is None:
            s, d, w = to.parse_edge_text(text)
            assert list(s) == [0] and list(w) == [2.0]
            continue
        with pytest.raises(to.TextError) as e:
            to.parse_edge_text(text)
        assert (e.value.kind, e.value.edge) == (kind, edge)


@pytest.mark.parametrize("name", text_cases.cases())
def test_c_oracle_reads_like_the_reference(name):
    text, want = text_cases.load(name)
    if isinstance(want, str):
        with pytest.raises(to.TextError) as e:
            to.parse_edge_text_c(text)
        assert e.value.kind == "weight"
        return
    got = to.csr_from_edges_c(*to.parse_edge_text_c(text))
    assert all(np.array_equal(a, b) for a, b in zip(got, want))


def test_c_oracle_matches_python_oracle():
    rng = np.random.default_rng(9)
    toks = [b"0", b"17", b"+3", b"-2", b"1.5", b"2.", b".5e1", b"1e400", b"1e-400", b"x", b"00",
            b"3e", b"99999999999", b"4.0000000000000000000000001"]
    for trial in range(300):
        k = int(rng.integers(0, 40))
        parts = [toks[i] for i in rng.integers(0, len(toks), k)]
        seps = [(b" ", b"\n", b"\t", b"\r\n")[i] for i in rng.integers(0, 4, k)]
        text = b"".join(p + s for p, s in zip(parts, seps))
        outs = []
        for f in (to.parse_edge_text, to.parse_edge_text_c):
            try:
                outs.append(tuple(a.tolist() for a in f(text)))
            except to.TextError as e:
                outs.append((e.kind, e.edge))
        assert outs[0] == outs[1], text


def test_edge_list_text_formatter():
    """graphs.EdgeList.text() (array formatting of the bench's text workload) writes exactly the
    "src dst w" lines a plain formatter writes, and the text oracle reads them back."""
    import graphs

    for el in (graphs.road_grid(48, 40, seed=3), graphs.rgg_knn(3000, seed=2)):
        want = b"".join(b"%d %d %d\n" % (a, b, c) for a, b, c in zip(el.src, el.dst, el.w))
        text = el.text()
        assert text == want
        s, d, w = to.parse_edge_text_c(text)
        assert np.array_equal(s, el.src) and np.array_equal(d, el.dst) and np.array_equal(w, el.w)

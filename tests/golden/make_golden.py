"""Regenerate the golden fixtures of tests/golden from the reference itself.

Runs the reference fast-bc headers (compiled in place by ``make -C oracle ref`` into
oracle/_ref/ref_harness) single-threaded on the seeded workloads and stores:
  grid32_exact_bc.txt        ExactBrandesBC<int,double> over the 32x32 grid (%.17g)
  grid32_ss.npz              DijkstraSSBrandesBC dependency vectors for a few sources
  grid256_clustered.npz      the clustered run on the 256x256 grid (Louvain seeds 1-4,
                             precision 0.01, kfrac 0.5): partition, borders, pivots and
                             cardinalities, intra-cluster BC, final BC (step replay and the
                             reference's own ClusteredBrandeBC::computeBC)
  grid256_classes.npz        VertexInfoPivotSelector (the exact topological classes) on every
                             cluster of that partition after DijkstraClusterEvaluator: class
                             offsets, pivots, cardinalities, and the intra-cluster BC it compared
  grid2048_partition.npz     LouvainGraphPartition (seeds 1-4, precision 0.01) of the
                             2048x2048 grid: community id per vertex (int16; every
                             community's vertices are ascending, as the reference lists them)
  grid2048_pivots.npz        KMeansPivotSelector (kfrac 0.5) on three communities of that partition
                             (5,220, 9,150 and 13,813 vertices), from the oracle's intra-cluster BC
                             and border vectors: pivots and cardinalities per community
  DWGtext.txt                the reference unit tests' 9-vertex fixture (copied)
  rgg1500_exact_bc.txt       ExactBrandesBC<int,double> over a 1,500-point random geometric graph
                             (3-NN, weights ceil(1000 d): the family of the 48-graph batch)
  rgg1500_ss.npz             DijkstraSSBrandesBC dependency vectors on it for three sources
  rgg1500_cluster.npz        DijkstraClusterEvaluator on its cluster of ids 0..499: intra BC,
                             borders, border lengths and counts
  text/<case>.txt, .out      edge-list texts in the formats operator>> accepts (layout, number
                             forms, weights past a double's fast conversion, overflow ending the
                             reading, rejected weights) and what DirectedWeightedGraph(istream&)
                             made of each: "n m" and the forward stars, or "error <what()>"
The clustered run takes about 15 minutes on one core, the 2048x2048 partition about a
minute on eight.  Usage:
  python tests/golden/make_golden.py [--reuse DIR]   (DIR: outputs of an earlier harness run)
  python tests/golden/make_golden.py --only text     (the text/ fixtures alone, seconds)
  python tests/golden/make_golden.py --only rgg      (the random-geometric-graph golden, seconds)
  python tests/golden/make_golden.py --only c5pivots [--reuse DIR]
                                                     (grid2048_pivots.npz: the reference's k-means
                                                     pivot sets of three communities of the 2048x2048
                                                     grid; hours, the communities in parallel)
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("FASTBC_REF_DIR", "")  # the reference checkout; required
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
sys.path.insert(0, os.path.join(ROOT, "fast-bc_gb300"))
import graphs  # noqa: E402

ENV = dict(os.environ, OMP_NUM_THREADS="1")


def run(*args, cwd=None):
    subprocess.run([HARNESS, *map(str, args)], check=True, env=ENV, cwd=cwd)


def parse_clusters(path):
    with open(path) as f:
        lines = f.read().split("\n")
    nc = int(lines[0])
    cv, bv, pv, kv = [], [], [], []
    for c in range(nc):
        rows = [list(map(int, lines[1 + 4 * c + k].split())) for k in range(4)]
        for dst, r in zip((cv, bv, pv, kv), rows):
            assert r[0] == len(r) - 1
            dst.append(np.array(r[1:], np.int32))
    def flat(lst):
        off = np.zeros(len(lst) + 1, np.int64)
        off[1:] = np.cumsum([x.size for x in lst])
        return off, (np.concatenate(lst) if lst else np.zeros(0, np.int32)).astype(np.int32)
    return flat(cv), flat(bv), flat(pv), flat(kv)


def text_cases() -> dict:
    """Edge-list texts whose reading is defined by the reference parser (every merged weight an
    integer, which the GPU engine requires)."""
    rng = np.random.default_rng(11)
    cases = {
        # tabs, runs of spaces, CRLF, blank lines, leading spaces, no final newline
        "layout": b"  0 1 3\r\n1\t2\t4\n\n\n2   0 5\r\n\t 0 2 1\n1 0\t\t2",
        # signs, leading zeros, points, exponents; repeated pairs summed (2.5 + 0.5, 10 + 2.5 + 0.5)
        "numbers": (b"+0 1 +3\n001 2 3.\n2 0 .5e1\n0 2 2.50\n0 2 0.5\n1 0 1E+1\n1 0 250e-2\n"
                    b"1 0 0.5\n2 1 0000.000100e4\n-0 3 7000e-3\n3 0 +.2e1\n"),
        # more than 19 significant digits or powers of ten past 10^22
        "long_weights": (b"0 1 1.0000000000000000000000001\n1 2 3000000000000000000000000000e-27\n"
                         b"2 0 0.000000000000000000000000000000000000000007e42\n"
                         b"0 2 2.99999999999999999999999999999\n2 1 40000000000000000000000e-22\n"
                         b"1 0 6.000000000000000000000000000001\n1 1 1e0000000000000000000000000\n"),
        # a weight past the largest double ends the reading; what follows is never read
        "overflow_stops": b"0 1 2\n1 0 3\n1 0 1e400\n2 1 oops\n",
        "zero_weight": b"0 1 2\n1 0 0\n1 1 1\n",
        "negative_weight": b"0 1 2\n1 0 -3\n",
        "word_weight": b"0 1 2\n1 0 abc\n",
        "underflow_weight": b"0 1 2\n1 0 1e-400\n",
    }
    # a few thousand edges over 300 vertices, repeated pairs, random spacing and integer
    # weights written in assorted forms
    n, m = 300, 4000
    src = rng.integers(0, n, m)
    dst = rng.integers(0, n, m)
    src[:n] = np.arange(n)  # every id a source, so n = 300
    w = rng.integers(1, 50, m)
    forms = [lambda x: b"%d" % x, lambda x: b"%d.0" % x, lambda x: b"+%d" % x,
             lambda x: b"%.1fe1" % (x / 10), lambda x: b"%de-1" % (10 * x),
             lambda x: b"%d.000000000000000000001" % x, lambda x: b"0%d." % x]
    seps = [b" ", b"\t", b"  ", b" \t "]
    ends = [b"\n", b"\r\n", b"\n\n", b" \n"]
    out = []
    for i in range(m):
        f = forms[rng.integers(len(forms))]
        sp = seps[rng.integers(len(seps))]
        out.append(b"%d%s%d%s%s%s" % (src[i], sp, dst[i], sp, f(int(w[i])), ends[rng.integers(len(ends))]))
    cases["mixed"] = b"".join(out)
    return cases


def rgg_golden() -> None:
    work = tempfile.mkdtemp()
    p = os.path.join(work, "rgg1500.txt")
    graphs.rgg_knn(1500, seed=11).write(p)
    run("exact", p, os.path.join(HERE, "rgg1500_exact_bc.txt"))
    srcs = [0, 700, 1499]
    deps = []
    for s in srcs:
        o = os.path.join(work, f"ss{s}.txt")
        run("ss", p, s, o)
        deps.append(np.loadtxt(o))
    np.savez_compressed(os.path.join(HERE, "rgg1500_ss.npz"), sources=np.array(srcs), dep=np.array(deps))
    # DijkstraClusterEvaluator on the cluster of ids 0..499 (spatially scattered: most members
    # are borders, and many borders are unreachable from a member)
    vf = os.path.join(work, "verts.txt")
    with open(vf, "w") as f:
        f.write(" ".join(str(v) for v in range(500)))
    pre = os.path.join(work, "clu")
    run("cluster", p, vf, pre)
    bc = np.loadtxt(pre + ".bc")
    with open(pre + ".vi") as f:
        lines = f.read().split("\n")
    nb = int(lines[0])
    borders = np.array(lines[1].split(), np.int32) if nb else np.zeros(0, np.int32)
    vals = [np.array(lines[2 + i].split(), np.float64).reshape(nb, 2) if nb else np.zeros((0, 2))
            for i in range(500)]
    np.savez_compressed(os.path.join(HERE, "rgg1500_cluster.npz"), intra_bc=bc, borders=borders,
                        border_len=np.array([v[:, 0] for v in vals]), border_cnt=np.array([v[:, 1] for v in vals]))


# Communities of the 2048x2048 grid's reference partition whose reference pivot sets are stored:
# about the 10th, 25th and 50th percentile of the 290 communities with borders (5,220, 9,150 and
# 13,813 vertices).  All 290 are out of reach: the reference's k-means with kfrac 0.5 runs
# O(classes * k * borders) per Lloyd step, and a median community has 13,577 exact classes
# (k = 6,788) over 544 borders.
C5_CLUSTERS = (124, 199, 78)


def c5_cluster_file(work: str, c: int, el, og, cid, isb) -> str:
    """The oracle's DijkstraClusterEvaluator restatement (one thread: the intra BC bit-identical to
    the reference's) on community c: vertices, intra BC, border lengths and counts in the binary
    layout of ref_harness select."""
    import oracle

    fn = os.path.join(work, f"c{c}.bin")
    if os.path.exists(fn):
        return fn
    vs = np.nonzero(cid == c)[0].astype(np.int32)
    bs = vs[isb[vs]]
    acc = np.zeros(el.n)
    _, bd, bsg = oracle.cluster_eval(og, vs, bs, acc, threads=1)
    with open(fn + ".tmp", "wb") as f:
        f.write(np.array([vs.size, bs.size], np.int64).tobytes())
        for a in (vs, acc[vs], bd, bsg):
            f.write(np.ascontiguousarray(a).tobytes())
    os.replace(fn + ".tmp", fn)
    return fn


def _unlimited_stack():
    import resource

    resource.setrlimit(resource.RLIMIT_STACK, (resource.RLIM_INFINITY, resource.RLIM_INFINITY))


def _c5_select(args) -> str:
    """ref_harness select on one community (KMeansPivotSelector, kfrac 0.5, one thread).  The
    reference's OpenMP array reduction in PlusPlusKMeans::computeCentroids keeps a private copy on
    the stack, which overflows the default 8 MB on these communities: the stack is unlimited."""
    txt, fn, out = args
    if not os.path.exists(out):
        with open(out + ".tmp", "w") as f:
            subprocess.run([HARNESS, "select", txt, "0.5", fn], stdout=f, check=True, env=ENV,
                           preexec_fn=_unlimited_stack)
        os.replace(out + ".tmp", out)
    return out


def read_piv(path: str):
    with open(path) as f:
        a, b = f.read().split("\n")[:2]
    a = list(map(int, a.split()[1:]))
    b = list(map(int, b.split()))
    assert a[0] == len(a) - 1 == b[0] == len(b) - 1
    return np.array(a[1:], np.int32), np.array(b[1:], np.int32)


def c5_pivots(work: str) -> None:
    """grid2048_pivots.npz: the reference's pivot sets (KMeansPivotSelector over
    VertexInfoPivotSelector and PlusPlusKMeans, kfrac 0.5; KMeansPivotSelector.h:79-132) of the
    C5_CLUSTERS communities of the reference partition, from their intra-cluster BC and border
    vectors (the oracle, pinned bit-identical to DijkstraClusterEvaluator).  Up to hours per
    community; the communities run in parallel processes."""
    import multiprocessing as mp

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    el = graphs.WORKLOADS["grid2048"]()
    txt = os.path.join(work, "grid2048.txt")
    if not os.path.exists(txt):
        el.write(txt)
    rp, col, _ = el.csr()
    cid = np.load(os.path.join(HERE, "grid2048_partition.npz"))["community"].astype(np.int64)
    src = np.repeat(np.arange(el.n), np.diff(rp))
    cross = cid[src] != cid[col]
    isb = np.zeros(el.n, bool)
    isb[src[cross]] = True
    isb[col[cross]] = True
    og = oracle.CSR.from_edgelist(el)
    jobs = [(txt, c5_cluster_file(work, c, el, og, cid, isb), os.path.join(work, f"c{c}.piv"))
            for c in C5_CLUSTERS]
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        outs = pool.map(_c5_select, jobs)
    piv, crd = [], []
    for c, out in zip(C5_CLUSTERS, outs):
        p, k = read_piv(out)
        assert np.all(cid[p] == c) and int(k.sum()) == int(np.sum(cid == c))
        piv.append(p)
        crd.append(k)
    off = np.zeros(len(piv) + 1, np.int64)
    off[1:] = np.cumsum([p.size for p in piv])
    np.savez_compressed(os.path.join(HERE, "grid2048_pivots.npz"), clusters=np.array(C5_CLUSTERS, np.int32),
                        pivot_off=off, pivots=np.concatenate(piv), cards=np.concatenate(crd))


def text_goldens() -> None:
    tdir = os.path.join(HERE, "text")
    os.makedirs(tdir, exist_ok=True)
    for name, data in text_cases().items():
        p = os.path.join(tdir, name + ".txt")
        with open(p, "wb") as f:
            f.write(data)
        run("graph", p, os.path.join(tdir, name + ".out"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reuse", default=None)
    ap.add_argument("--only", choices=["text", "rgg", "c5pivots"], default=None)
    a = ap.parse_args()
    if not REF or not os.path.isdir(os.path.join(REF, "libfastbc")):
        sys.exit("set FASTBC_REF_DIR to the reference checkout")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"], check=True)
    if a.only == "c5pivots":
        work = a.reuse or tempfile.mkdtemp()
        os.makedirs(work, exist_ok=True)
        c5_pivots(work)
        return
    if a.only != "rgg":
        text_goldens()
    if a.only != "text":
        rgg_golden()
    if a.only:
        return
    shutil.copy(os.path.join(REF, "libfastbc", "test", "DWGtext.txt"), os.path.join(HERE, "DWGtext.txt"))
    work = a.reuse or tempfile.mkdtemp()
    g32 = os.path.join(work, "grid32.txt")
    g256 = os.path.join(work, "grid256.txt")
    if not os.path.exists(g32):
        graphs.WORKLOADS["grid32"]().write(g32)
    if not os.path.exists(g256):
        graphs.WORKLOADS["grid256"]().write(g256)
    run("exact", g32, os.path.join(HERE, "grid32_exact_bc.txt"))
    srcs = [0, 77, 512, 1023]
    deps = []
    for s in srcs:
        out = os.path.join(work, f"ss{s}.txt")
        run("ss", g32, s, out)
        deps.append(np.loadtxt(out))
    np.savez_compressed(os.path.join(HERE, "grid32_ss.npz"), sources=np.array(srcs), dep=np.array(deps))
    pre = os.path.join(work, "grid256")
    if not os.path.exists(pre + ".bc_ref"):
        run("clustered", g256, "1,2,3,4", 0.01, 0.5, pre)
    (coff, cv), (boff, bv), (poff, pv), (koff, kv) = parse_clusters(pre + ".clusters")
    assert np.array_equal(poff, koff)
    bc = np.loadtxt(pre + ".bc")
    bc_ref = np.loadtxt(pre + ".bc_ref")
    # the replay adds straight into globalBC; computeBC's one-thread OpenMP reduction adds a
    # private sum at the end, so the two agree to rounding only
    assert np.max(np.abs(bc - bc_ref)) <= 1e-12 * np.max(np.abs(bc_ref)), "replay != computeBC"
    np.savez_compressed(os.path.join(HERE, "grid256_clustered.npz"), cluster_off=coff,
                        cluster_vertices=cv, border_off=boff, borders=bv, pivot_off=poff,
                        pivots=pv, cards=kv, intra_bc=np.loadtxt(pre + ".intra"), bc=bc_ref,
                        bc_replay=bc)
    clu = os.path.join(work, "grid256.clu")
    with open(clu, "w") as f:
        for c in range(coff.size - 1):
            vs = cv[coff[c]:coff[c + 1]]
            f.write(f"{vs.size} " + " ".join(map(str, vs)) + "\n")
    cls = os.path.join(work, "grid256cls")
    subprocess.run([HARNESS, "classes", g256, clu, cls], check=True, env=dict(os.environ, OMP_NUM_THREADS="8"))
    with open(cls + ".classes") as f:
        lines = f.read().split("\n")
    piv, crd = [], []
    for c in range(coff.size - 1):
        a = list(map(int, lines[2 * c].split()))
        b = list(map(int, lines[2 * c + 1].split()))
        assert a[0] == len(a) - 1 == b[0] == len(b) - 1
        piv.append(np.array(a[1:], np.int32))
        crd.append(np.array(b[1:], np.int32))
    class_off = np.zeros(len(piv) + 1, np.int64)
    class_off[1:] = np.cumsum([p.size for p in piv])
    # the BC the selector compared is stored with it (OpenMP reductions round differently)
    np.savez_compressed(os.path.join(HERE, "grid256_classes.npz"), class_off=class_off,
                        pivots=np.concatenate(piv), cards=np.concatenate(crd),
                        intra_bc=np.loadtxt(cls + ".intra"))
    g2048 = os.path.join(work, "grid2048.txt")
    if not os.path.exists(g2048):
        graphs.WORKLOADS["grid2048"]().write(g2048)
    part = os.path.join(work, "grid2048.part")
    if not os.path.exists(part):
        subprocess.run([HARNESS, "partition", g2048, "1,2,3,4", "0.01", part], check=True,
                       env=dict(os.environ, OMP_NUM_THREADS="8"))
    with open(part) as f:
        lines = f.read().split("\n")
    comms = [np.array(lines[1 + i].split()[1:], np.int32) for i in range(int(lines[0]))]
    cid = np.full(sum(c.size for c in comms), -1, np.int16)
    for i, c in enumerate(comms):
        assert np.all(np.diff(c) > 0)
        cid[c] = i
    assert np.all(cid >= 0)
    np.savez_compressed(os.path.join(HERE, "grid2048_partition.npz"), community=cid)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()

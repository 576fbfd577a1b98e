"""Edge-list text reading -- TEST INFRASTRUCTURE ONLY (the checker of fbc_graph_from_text).

A restatement of DirectedWeightedGraph(std::istream&) (DirectedWeightedGraph.h:67-96) and of
addEdge (DirectedWeightedGraph.h:136-170) for well-formed input:
  * the text is read as whitespace-separated triples "src dst weight" (operator>> skips the
    C locale's spaces: space, \\t, \\n, \\v, \\f, \\r -- the set bytes.split() uses);
  * src and dst are decimal ints ([+-]?[0-9]+ within int32);
  * the weight is a decimal double ([+-]?(digits[.digits] | .digits)([eE][+-]?digits)?),
    correctly rounded (libstdc++ hands the token to strtod; Python's float() rounds the same
    way); a weight that overflows a double makes operator>> fail with the largest double, which
    passes the weight check, and the loop ends before that edge (DirectedWeightedGraph.h:78-86);
    a weight <= 0 -- including a token that is not a number, read as 0 -- throws
    std::invalid_argument("Edge weight must be greater than zero");
  * repeated (src, dst) pairs have their weights summed in input order, rows ascend by
    destination (std::map), and n = 1 + the largest source id.
Cases the reference leaves undefined (an id token that is not an int, text ending inside a
triple) raise TextError here, as fbc_graph_from_text reports them.
Pinned against the reference's own parser on the fixtures in tests/golden/text/.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import re

import numpy as np

_INT = re.compile(rb"[+-]?[0-9]+\Z")
_DBL = re.compile(rb"[+-]?(?:[0-9]+\.?[0-9]*|\.[0-9]+)(?:[eE][+-]?[0-9]+)?\Z")


class TextError(ValueError):
    """kind: 'weight' (<= 0 or not a number), 'id' (not a decimal int32) or 'incomplete'."""

    def __init__(self, kind: str, edge: int):
        super().__init__(f"{kind} at edge {edge}")
        self.kind = kind
        self.edge = edge


def _int32(tok: bytes, e: int) -> int:
    if not _INT.match(tok):
        raise TextError("id", e)
    v = int(tok)
    if not -(1 << 31) <= v < (1 << 31):
        raise TextError("id", e)
    return v


def parse_edge_text(data: bytes):
    """(src int32, dst int32, w float64) of the edges the reference reads from `data`."""
    toks = bytes(data).split()
    ne = len(toks) // 3
    src, dst, w = [], [], []
    for e in range(ne):
        s, d, x = toks[3 * e:3 * e + 3]
        a, b = _int32(s, e), _int32(d, e)
        if not _DBL.match(x):
            raise TextError("weight", e)
        v = float(x)
        if math.isinf(v) and v > 0:
            break  # the reading ends here
        if not v > 0:
            raise TextError("weight", e)
        src.append(a)
        dst.append(b)
        w.append(v)
    else:
        if len(toks) % 3:
            raise TextError("incomplete", ne)
    return np.array(src, np.int32), np.array(dst, np.int32), np.array(w, np.float64)


def csr_from_edges(src, dst, w):
    """(row_ptr int64, col int32, w float64): addEdge's merge of repeated pairs (weights summed in
    input order) and the forward stars in ascending destination order."""
    src = np.asarray(src, np.int64)
    dst = np.asarray(dst, np.int64)
    n = int(src.max()) + 1 if src.size else 0
    order = np.lexsort((dst, src))  # stable: input order within a pair
    col, ww = [], []
    rp = np.zeros(n + 1, np.int64)
    prev = None
    for i in order:
        key = (int(src[i]), int(dst[i]))
        if key == prev:
            ww[-1] += float(w[i])
        else:
            col.append(key[1])
            ww.append(float(w[i]))
            rp[key[0] + 1] += 1
            prev = key
    return np.cumsum(rp), np.array(col, np.int32), np.array(ww, np.float64)


# the same reading in C (text_oracle.c, in liboracle.so): fast enough for full-size texts and
# for the CPU baseline of the device parser
_KINDS = {1: "weight", 2: "id", 3: "incomplete"}
_clib = None


def _c():
    global _clib
    if _clib is None:
        lib = C.CDLL(os.path.join(os.path.dirname(os.path.abspath(__file__)), "liboracle.so"))
        i64, vp = C.c_int64, C.c_void_p
        lib.orc_parse_text.argtypes = [C.c_char_p, i64, vp, vp, vp, i64, C.POINTER(i64), C.POINTER(i64)]
        lib.orc_parse_text.restype = C.c_int
        lib.orc_csr_from_edges.argtypes = [i64, vp, vp, vp, C.c_int32, vp, vp, vp]
        lib.orc_csr_from_edges.restype = i64
        _clib = lib
    return _clib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def parse_edge_text_c(data: bytes):
    data = bytes(data)
    cap = max(1, data.count(b"\n") + 1, len(data) // 6 + 1)  # every edge needs at least 6 bytes
    src = np.empty(cap, np.int32)
    dst = np.empty(cap, np.int32)
    w = np.empty(cap, np.float64)
    cnt, edge = C.c_int64(), C.c_int64()
    rc = _c().orc_parse_text(data, len(data), _p(src), _p(dst), _p(w), cap, C.byref(cnt), C.byref(edge))
    if rc != 0:
        if rc < 0:
            raise MemoryError("edge capacity")
        raise TextError(_KINDS[rc], int(edge.value))
    k = int(cnt.value)
    return src[:k], dst[:k], w[:k]


def csr_from_edges_c(src, dst, w):
    src = np.ascontiguousarray(src, np.int32)
    dst = np.ascontiguousarray(dst, np.int32)
    w = np.ascontiguousarray(w, np.float64)
    n = int(src.max()) + 1 if src.size else 0
    rp = np.zeros(n + 1, np.int64)
    col = np.empty(max(src.size, 1), np.int32)
    ww = np.empty(max(src.size, 1), np.float64)
    m = _c().orc_csr_from_edges(src.size, _p(src), _p(dst), _p(w), n, _p(rp), _p(col), _p(ww))
    assert m >= 0
    return rp, col[:m], ww[:m]

"""The edge-list text fixtures of tests/golden/text: each <case>.txt with what the reference's
parser made of it (<case>.out: "n m" and the forward stars, or "error <message>")."""
import os

import numpy as np

from conftest import GOLDEN

TEXT_DIR = os.path.join(GOLDEN, "text")


def cases():
    return sorted(f[:-4] for f in os.listdir(TEXT_DIR) if f.endswith(".txt"))


def load(name):
    """(text bytes, expected) with expected = (rp, col, w) or the error message."""
    with open(os.path.join(TEXT_DIR, name + ".txt"), "rb") as f:
        text = f.read()
    with open(os.path.join(TEXT_DIR, name + ".out")) as f:
        lines = f.read().splitlines()
    if lines[0].startswith("error "):
        return text, lines[0][6:]
    n, m = map(int, lines[0].split())
    rows = [ln.split() for ln in lines[1:]]
    assert len(rows) == m
    src = np.array([int(r[0]) for r in rows], np.int64)
    col = np.array([int(r[1]) for r in rows], np.int32)
    w = np.array([float(r[2]) for r in rows], np.float64)
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, src + 1, 1)
    return text, (np.cumsum(rp), col, w)

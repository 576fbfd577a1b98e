"""Every `File.h:a-b` / `File.cpp:a` citation of the reference in this repository's sources and
notes points inside an existing reference file (CPU; skipped where the reference tree is absent)."""
import os
import re

import pytest

from conftest import ROOT

REF = os.environ.get("FASTBC_REF_DIR", "")  # the reference checkout (unset: skipped)
CITE = re.compile(r"\b([A-Za-z_]+\.(?:h|cpp)):(\d+)(?:-(\d+))?")
SKIP_DIRS = ("_work", ".git", "gpurun_out", "baseline", "_ref", "__pycache__")


def test_reference_citations_in_range():
    if not REF or not os.path.isdir(REF):
        pytest.skip("reference tree not given (FASTBC_REF_DIR)")
    lengths = {}
    for root, _, files in os.walk(REF):
        for f in files:
            if f.endswith((".h", ".cpp")):
                with open(os.path.join(root, f), errors="replace") as fh:
                    n = sum(1 for _ in fh)
                lengths[f] = max(lengths.get(f, 0), n)
    bad, seen = [], 0
    for root, dirs, files in os.walk(ROOT):
        dirs[:] = [d for d in dirs if d not in SKIP_DIRS]
        for f in files:
            if not f.endswith((".py", ".cu", ".cuh", ".h", ".hpp", ".c", ".cpp", ".md")):
                continue
            path = os.path.join(root, f)
            with open(path, errors="replace") as fh:
                for i, line in enumerate(fh, 1):
                    for m in CITE.finditer(line):
                        name, a = m.group(1), int(m.group(2))
                        b = int(m.group(3) or a)
                        if name not in lengths:
                            continue
                        seen += 1
                        if a > b or b > lengths[name]:
                            bad.append(f"{os.path.relpath(path, ROOT)}:{i}: {m.group(0)} ({name} has {lengths[name]} lines)")
    assert seen > 100
    assert not bad, "\n".join(bad)

"""The result file of the fbc CLI (main.cpp:123-130, 282-294), written by the Python binding and
by the C++ layer: the same bytes as the reference's `outFile << bc[i] << std::endl` (six
significant digits; negatives and NaN written as 0) and an existing file refused (CPU only)."""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

VALUES = [2.0, 4.333333333333333, 1.3333333333333333, 7.6666666666666661, -1e-12, 0.0, 123456789.0,
          1e-7, 0.000123456789, 65535.5, 1e21, math.nan, -0.0]


def test_python_writer(tmp_path):
    import fastbc_gpu as fg

    p = tmp_path / "bc.txt"
    fg.write_bc(str(p), np.array(VALUES))
    lines = p.read_text().splitlines()
    assert lines[:4] == ["2", "4.33333", "1.33333", "7.66667"]
    assert lines[4] == "0" and lines[6] == "1.23457e+08" and lines[7] == "1e-07" and lines[11] == "0"
    with pytest.raises(FileExistsError):
        fg.write_bc(str(p), np.array(VALUES))


def test_cpp_writer_matches_python(tmp_path):
    import fastbc_gpu as fg

    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    vals = ", ".join(repr(v) if not math.isnan(v) else "std::nan(\"\")" for v in VALUES)
    src = tmp_path / "w.cpp"
    src.write_text('#include <cmath>\n#include "fastbc_gpu/engine.hpp"\nint main(int, char** argv) {\n'
                   f"    std::vector<double> bc{{{vals}}};\n    fbcgpu::write_bc(argv[1], bc);\n"
                   "    try { fbcgpu::write_bc(argv[1], bc); } catch (const fbcgpu::Error&) { return 0; }\n"
                   "    return 1;\n}\n")
    exe = tmp_path / "w"
    lib = os.path.join(ROOT, "fast-bc_gb300")
    r = subprocess.run([gxx, "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-L", lib, "-lfbcgpu",
                        "-Wl,-rpath," + lib, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out_cpp = tmp_path / "cpp.txt"
    r = subprocess.run([str(exe), str(out_cpp)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out_py = tmp_path / "py.txt"
    fg.write_bc(str(out_py), np.array(VALUES))
    assert out_cpp.read_bytes() == out_py.read_bytes()

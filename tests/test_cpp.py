"""The C++ layer over the C ABI.

* test_adapters_compile_against_reference (CPU): the drop-in classes of
  include/fastbc_gpu/fastbc_adapters.hpp compile and link against the reference's own interface
  headers (skipped where the reference tree is absent, e.g. on the GPU machine).
* test_reference_unit_tests_restated (GPU): tests/cpp/brandes_tests.cpp, the reference's
  Brandes unit tests (ExactBrandesBC.cpp, DijkstraClusterEvaluator.cpp, DijkstraSSBrandesBC.cpp)
  restated against include/fastbc_gpu/engine.hpp, built with g++ and run on the GPU.
"""
import os
import shutil
import subprocess

import pytest

from conftest import GOLDEN, ROOT

REF = os.environ.get("FASTBC_REF_DIR", "")  # the reference checkout (unset: skipped)
LIBDIR = os.path.join(ROOT, "fast-bc_gb300")


def _gxx():
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    return gxx


def test_adapters_compile_against_reference(tmp_path):
    gxx = _gxx()
    if not os.path.isdir(os.path.join(REF, "libfastbc", "include")):
        pytest.skip("reference headers not present")
    out = tmp_path / "adapter_compile.o"
    cmd = [gxx, "-std=c++17", "-fopenmp", "-w", "-c",
           "-DFASTBC_BRANDES_ENABLE_PIVOT_BORDER", "-DFASTBC_BRANDES_CLUSTERED_IGNORE_UNCONNECTED",
           "-I", os.path.join(ROOT, "oracle", "ref_stub"), "-I", os.path.join(REF, "libfastbc", "include"),
           "-I", os.path.join(ROOT, "include"),
           "-include", "limits", "-include", "stdexcept", "-include", "set", "-include", "map",
           "-include", "sstream",
           os.path.join(ROOT, "tests", "cpp", "adapter_compile.cpp"), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.gpu
def test_reference_unit_tests_restated(fg, tmp_path):
    gxx = _gxx()
    exe = tmp_path / "brandes_tests"
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "brandes_tests.cpp"), "-L", LIBDIR, "-lfbcgpu",
                        "-Wl,-rpath," + LIBDIR, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([str(exe), os.path.join(GOLDEN, "DWGtext.txt")], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "all passed" in r.stdout

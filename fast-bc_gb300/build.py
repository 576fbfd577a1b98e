"""Build the GB300 engine in place: one nvcc translation unit for sm_103a -> libfbcgpu.so.

The library links the CUDA runtime statically and has no PyTorch dependency; its C ABI is
declared in include/fbc_gpu.h.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = [os.path.join(HERE, "csrc", "fbc_gpu.cu"), os.path.join(HERE, "csrc", "noalloc.cu")]
HEADERS = sorted(os.path.join(HERE, "csrc", f) for f in os.listdir(os.path.join(HERE, "csrc"))
                 if f.endswith(".cuh")) + [os.path.join(ROOT, "include", "fbc_gpu.h")]
OUT = os.path.join(HERE, "libfbcgpu.so")


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if force or _stale(OUT, SOURCES + HEADERS):
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
               "-I", os.path.join(ROOT, "include"), *SOURCES, "-o", OUT + ".tmp"]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        subprocess.run(cmd, check=True)
        os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    build(force=True, verbose=True)

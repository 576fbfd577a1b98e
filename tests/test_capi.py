"""The C ABI library loads and exports every entry point include/fbc_gpu.h declares (CPU only:
no compute call is made; without a GPU fbc_gpu_init reports a CUDA error)."""
import ctypes as C
import os
import re

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "fbc_gpu.h")
LIB = os.path.join(ROOT, "fast-bc_gb300", "libfbcgpu.so")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fbc_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = declared()
    for must in ("fbc_gpu_init", "fbc_exact_bc", "fbc_single_source", "fbc_sssp_dependency_batch",
                 "fbc_cluster_eval_batch", "fbc_multi_exact_bc", "fbc_sssp_debug", "fbc_last_error_string"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(LIB)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_calls_fail_cleanly_before_init():
    lib = C.CDLL(LIB)
    lib.fbc_last_error_string.restype = C.c_char_p
    out = C.c_void_p()
    rp = (C.c_int64 * 2)(0, 0)
    rc = lib.fbc_graph_upload(1, rp, None, None, C.byref(out))
    assert rc in (7, 2)  # FBC_ERR_NOT_INIT (or a CUDA error where no driver is present)
    assert lib.fbc_last_error_string()


def test_header_is_plain_c(tmp_path):
    """A C program (no C++) includes the header without warnings and links every entry point."""
    import shutil
    import subprocess

    import pytest

    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc not available")
    calls = "\n".join(f"    (void)&{n};" for n in declared())
    src = tmp_path / "abi.c"
    src.write_text('#include "fbc_gpu.h"\nint main(void) {\n' + calls + "\n    return 0;\n}\n")
    r = subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                        os.path.join(ROOT, "include"), str(src), "-L", os.path.dirname(LIB), "-lfbcgpu",
                        "-o", str(tmp_path / "abi")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


OPTIONS = ["delta", "block_threads", "frontier_threads", "group", "chunk_max", "wide_n", "warp_max_n",
           "order_min_n", "iter_mult", "ws_budget_mb", "csr_device_min_m", "wide_threads", "debug_sched",
           "scratch_keep_mb", "wide_kv", "adj4", "bc_sweep", "pull_count", "source_order"]

# defaults the header documents (a fresh process reads them before anything sets an option)
DEFAULTS = {"wide_threads": 1024, "wide_kv": 1, "adj4": 1, "bc_sweep": 1, "pull_count": 1, "source_order": 1,
            "order_min_n": 65536, "scratch_keep_mb": 8192}


def test_options_round_trip_and_limits():
    """The tuning knobs (host state, no GPU needed): every key the header documents reads back
    what was set within its documented range, out-of-range values are clamped, a bad group or an
    unknown key is refused with FBC_ERR_INVALID_ARG."""
    lib = C.CDLL(LIB)
    lib.fbc_set_option.argtypes = [C.c_char_p, C.c_int64]
    lib.fbc_get_option.argtypes = [C.c_char_p, C.POINTER(C.c_int64)]
    src = open(HEADER).read()
    for k in OPTIONS:
        assert f'"{k}"' in src, k
    saved = {}
    for k in OPTIONS:
        v = C.c_int64()
        assert lib.fbc_get_option(k.encode(), C.byref(v)) == 0
        saved[k] = v.value

    def get(k):
        v = C.c_int64()
        assert lib.fbc_get_option(k.encode(), C.byref(v)) == 0
        return v.value

    try:
        for k, v in [("delta", 37), ("chunk_max", 64), ("group", 2), ("order_min_n", 0), ("iter_mult", 3),
                     ("pull_count", 0), ("source_order", 0), ("bc_sweep", 0), ("adj4", 0), ("wide_kv", 2)]:
            assert lib.fbc_set_option(k.encode(), v) == 0 and get(k) == v
        assert lib.fbc_set_option(b"block_threads", 5000) == 0 and get("block_threads") == 1024
        assert lib.fbc_set_option(b"frontier_threads", 1) == 0 and get("frontier_threads") == 32
        assert lib.fbc_set_option(b"wide_threads", 300) == 0 and get("wide_threads") == 288
        assert lib.fbc_set_option(b"delta", -5) == 0 and get("delta") == 0
        assert lib.fbc_set_option(b"group", 3) == 1
        assert lib.fbc_set_option(b"no_such_knob", 1) == 1
        v = C.c_int64()
        assert lib.fbc_get_option(b"no_such_knob", C.byref(v)) == 1
    finally:
        for k, v in saved.items():
            lib.fbc_set_option(k.encode(), v)


def test_option_defaults():
    """A freshly loaded library reports the defaults the header documents."""
    import json
    import subprocess
    import sys

    code = ("import ctypes as C, json, sys\n"
            "lib = C.CDLL(sys.argv[1])\n"
            "lib.fbc_get_option.argtypes = [C.c_char_p, C.POINTER(C.c_int64)]\n"
            "out = {}\n"
            "for k in sys.argv[2:]:\n"
            "    v = C.c_int64()\n"
            "    assert lib.fbc_get_option(k.encode(), C.byref(v)) == 0\n"
            "    out[k] = v.value\n"
            "print(json.dumps(out))\n")
    r = subprocess.run([sys.executable, "-c", code, LIB, *DEFAULTS], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert json.loads(r.stdout) == DEFAULTS


def test_every_entry_point_refuses_cleanly_before_init():
    """Each entry point called before fbc_gpu_init with zero sizes and null pointers returns a
    status (FBC_ERR_NOT_INIT, or FBC_ERR_INVALID_ARG where the arguments are checked first; OK for
    the no-op frees) instead of dereferencing anything (CPU: the library never initialises here)."""
    import fastbc_gpu as fg

    skip = {"fbc_gpu_init", "fbc_last_error_string", "fbc_set_option", "fbc_get_option"}
    for name, (args, res) in sorted(fg.lib.signatures.items()):
        if name in skip:
            continue
        vals = [None if a in (C.c_void_p, C.c_char_p) or hasattr(a, "contents") else 0 for a in args]
        rc = getattr(fg.lib, name)(*vals)
        assert rc in (0, fg.FBC_ERR_INVALID_ARG, fg.FBC_ERR_NOT_INIT), (name, rc)
        if name in ("fbc_graph_free", "fbc_plan_free", "fbc_gpu_shutdown"):
            assert rc == 0, name

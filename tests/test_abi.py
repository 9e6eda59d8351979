"""The C ABI library: builds, loads and exports every entry point the header declares."""
import ctypes
import os
import re
import subprocess

from pyprop_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "pyprop_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pg_\w+)\s*\(", text)))


def test_library_exports_header_symbols():
    lib = _native.load()
    names = header_functions()
    assert len(names) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", _native.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (pg_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)
    # the Python binding covers the header
    assert set(_native.exported_symbols()) <= set(names)


def test_error_strings_and_version():
    lib = _native.load()
    assert lib.pg_error_string(0) == b"PG_OK"
    assert b"PG_ERR_SHAPE" in lib.pg_error_string(-4)
    assert b"sm_103a" in lib.pg_version()


def test_null_arguments_rejected_without_device():
    lib = _native.load()
    assert lib.pg_ctx_create(0, None) == -1
    assert lib.pg_op_destroy(None) == -1
    assert lib.pg_banded_apply(None, 0, None) == -1
    assert lib.pg_tensor_multiply_diag_bandnh(None, 1, 13, 1.0, None, 1, 1, None, 1, 1, 6, None) == -1
    # the pAMP step's switches and statistics
    assert lib.pg_pamp_step(None, None, 0.01, None, 0, None) == -1
    assert lib.pg_pamp_set_fused(None, 1) == -1
    assert lib.pg_pamp_set_device_exp(None, 1) == -1
    assert lib.pg_pamp_set_barrier_probe(None, 1, 0) == -1
    assert lib.pg_pamp_last_stats(None, None) == -1


def test_header_compiles_as_c():
    src = '#include "pyprop_gpu.h"\nint main(void){ pg_ctx *c = 0; (void)c; return PG_OK; }\n'
    path = "/tmp/pg_header_check.c"
    with open(path, "w") as fh:
        fh.write(src)
    res = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-c", path,
                          "-o", "/tmp/pg_header_check.o"], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr

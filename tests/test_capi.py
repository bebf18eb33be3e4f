"""The C ABI library loads and exports every function include/gpufs_gb300.h
declares (CPU only: no CUDA call is made)."""
import ctypes
import os
import re

import gpufs_gb300

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "gpufs_gb300.h")


def declared_functions():
    src = open(HDR).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([a-z_][a-z0-9_]*)\s*\([^;{]*\)\s*;", src)
    return sorted(set(n for n in names if n.startswith("gfs_")))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("gfs_create", "gfs_destroy", "gfs_run_handler", "gfs_pread", "gfs_pwrite", "gfs_memcopy"):
        assert n in names


def test_library_exports_all_declared(built):
    lib = ctypes.CDLL(gpufs_gb300.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(built):
    assert set(declared_functions()) <= set(gpufs_gb300._SIGS)


def test_product_does_not_use_oracle():
    """The shipped package never imports or links the checker."""
    pkg = os.path.dirname(gpufs_gb300.__file__)
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".c", ".cpp")):
                txt = open(os.path.join(dirpath, f), errors="ignore").read()
                assert "import oracle" not in txt and "from oracle" not in txt and "liboracle" not in txt, f

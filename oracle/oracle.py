"""ctypes binding of oracle/oracle.c (and, when built, oracle/_ref).

TEST INFRASTRUCTURE ONLY: the checker the CUDA path is compared against.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SRC = os.path.join(REF_DIR, "ref_match_string.c")
REF_SO = os.path.join(REF_DIR, "libref_grep.so")
_ROOT = None


def reference_root():
    """Where the reference source tree is looked for: $GPUFS_REFERENCE, else
    the default of the build recipe (oracle/build_ref.sh).  It may be absent
    (machines that run the GPU tests have none); callers check."""
    global _ROOT
    if _ROOT is None:
        _ROOT = os.environ.get("GPUFS_REFERENCE") or subprocess.run(
            ["sh", os.path.join(HERE, "build_ref.sh"), "--print-root"], stdout=subprocess.PIPE,
            text=True, check=True).stdout.strip()
    return _ROOT


def build():
    """Compile oracle.c, and the reference-derived checker when available."""
    src = os.path.join(HERE, "oracle.c")
    if not os.path.exists(SO) or os.path.getmtime(SO) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-shared", "-fPIC", "-pthread", "-o", SO, src])
    if not os.path.exists(REF_SRC) and os.path.isdir(reference_root()):
        subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), reference_root()])
    if os.path.exists(REF_SRC) and (not os.path.exists(REF_SO) or os.path.getmtime(REF_SO) < os.path.getmtime(REF_SRC)):
        subprocess.check_call(["gcc", "-O2", "-shared", "-fPIC", "-pthread", "-o", REF_SO, REF_SRC])


_L = None
_R = None


def L():
    global _L
    if _L is None:
        build()
        lib = ctypes.CDLL(SO)
        u64, vp, i = ctypes.c_uint64, ctypes.c_void_p, ctypes.c_int
        lib.orc_xxh64.restype = u64
        lib.orc_xxh64.argtypes = [vp, ctypes.c_size_t, u64]
        lib.orc_grep_match_string.restype = i
        lib.orc_grep_match_string.argtypes = [ctypes.c_char_p, ctypes.c_char_p, i]
        lib.orc_grep_file_faithful_word.restype = ctypes.c_uint32
        lib.orc_grep_file_faithful_word.argtypes = [ctypes.c_char_p, vp, ctypes.c_size_t]
        lib.orc_grep_split_points.restype = ctypes.c_size_t
        lib.orc_grep_split_points.argtypes = [vp, ctypes.c_size_t, vp, ctypes.c_size_t]
        lib.orc_grep_tail_start.restype = ctypes.c_size_t
        lib.orc_grep_tail_start.argtypes = [vp, ctypes.c_size_t]
        for fn in ("orc_grep_counts_faithful",):
            getattr(lib, fn).argtypes = [vp, i, vp, vp, i, vp]
        for fn in ("orc_grep_counts_fast", "orc_grep_counts_refalgo"):
            getattr(lib, fn).argtypes = [vp, i, vp, vp, i, vp, i]
        lib.orc_gemv_f64.argtypes = [vp, vp, ctypes.c_long, ctypes.c_long, vp, vp, i]
        lib.orc_xxh64_many.argtypes = [vp, vp, i, vp, i]
        _L = lib
    return _L


def ref():
    """The reference's own match_string compiled for the host, or None."""
    global _R
    if _R is None:
        build()
        if not os.path.exists(REF_SO):
            return None
        r = ctypes.CDLL(REF_SO)
        r.ref_match_string.restype = ctypes.c_int
        r.ref_match_string.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
        if hasattr(r, "ref_grep_counts"):
            vp = ctypes.c_void_p
            r.ref_grep_counts.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_int, vp, ctypes.c_int]
        _R = r
    return _R


def ref_grep_counts(dict_bytes, files, nthreads=None):
    """The reference's own matcher driven through its window walk (CPU), or
    None when the reference-derived library was not built."""
    r = ref()
    if r is None or not hasattr(r, "ref_grep_counts"):
        return None
    d = np.ascontiguousarray(np.frombuffer(dict_bytes, dtype=np.uint8))
    nw = d.size // 32
    arrs, ptrs, sizes = _files_arrays(files)
    out = np.zeros((nw, len(arrs)), dtype=np.uint32)
    r.ref_grep_counts(d.ctypes.data, nw, ptrs, sizes, len(arrs), out.ctypes.data,
                      nthreads or max(1, os.cpu_count() or 1))
    return out


def xxh64(data, seed=0):
    a = np.frombuffer(data, dtype=np.uint8) if not isinstance(data, np.ndarray) else data
    a = np.ascontiguousarray(a)
    return int(L().orc_xxh64(a.ctypes.data if a.size else None, a.size, seed))


def match_string(word33, data):
    return L().orc_grep_match_string(word33, data, len(data))


def _files_arrays(files):
    arrs = [np.ascontiguousarray(np.frombuffer(f, dtype=np.uint8) if not isinstance(f, np.ndarray) else f)
            for f in files]
    ptrs = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
    sizes = (ctypes.c_uint64 * len(arrs))(*[a.size for a in arrs])
    return arrs, ptrs, sizes


def grep_counts(dict_bytes, files, mode="fast", nthreads=None):
    """counts[w, f] = occurrences of dictionary record w in file f."""
    d = np.ascontiguousarray(np.frombuffer(dict_bytes, dtype=np.uint8))
    nw = d.size // 32
    arrs, ptrs, sizes = _files_arrays(files)
    out = np.zeros((nw, len(arrs)), dtype=np.uint32)
    nt = nthreads or max(1, os.cpu_count() or 1)
    if mode == "fast":
        L().orc_grep_counts_fast(d.ctypes.data, nw, ptrs, sizes, len(arrs), out.ctypes.data, nt)
    elif mode == "faithful":
        L().orc_grep_counts_faithful(d.ctypes.data, nw, ptrs, sizes, len(arrs), out.ctypes.data)
    elif mode == "refalgo":
        L().orc_grep_counts_refalgo(d.ctypes.data, nw, ptrs, sizes, len(arrs), out.ctypes.data, nt)
    else:
        raise ValueError(mode)
    return out


def split_points(data):
    a = np.ascontiguousarray(np.frombuffer(data, dtype=np.uint8))
    n = L().orc_grep_split_points(a.ctypes.data, a.size, None, 0)
    out = np.zeros(max(1, n), dtype=np.uint64)
    L().orc_grep_split_points(a.ctypes.data, a.size, out.ctypes.data, n)
    return out[:n]


def tail_start(data):
    """Offset of the bytes the reference's chunk walk reads a second time
    (len(data) when there are none)."""
    a = np.ascontiguousarray(np.frombuffer(data, dtype=np.uint8))
    return int(L().orc_grep_tail_start(a.ctypes.data if a.size else None, a.size))


def gemv_f64(A, x, nthreads=None):
    A = np.ascontiguousarray(A, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    rows, cols = A.shape
    y = np.zeros(rows, dtype=np.float64)
    ay = np.zeros(rows, dtype=np.float64)
    L().orc_gemv_f64(A.ctypes.data, x.ctypes.data, rows, cols, y.ctypes.data, ay.ctypes.data,
                     nthreads or max(1, os.cpu_count() or 1))
    return y, ay


def xxh64_many(files, nthreads=None):
    arrs, ptrs, sizes = _files_arrays(files)
    out = np.zeros(len(arrs), dtype=np.uint64)
    L().orc_xxh64_many(ptrs, sizes, len(arrs), out.ctypes.data, nthreads or max(1, os.cpu_count() or 1))
    return [int(v) for v in out]

"""gpufs_gb300: a GB300-native GPU file-system layer (GPUfs device API over an
HBM buffer cache), driven from Python through its C ABI.

The product is native: libgpufs_gb300.so (CUDA, sm_103a) built in-tree by
gpufs_gb300.build.  This module only binds the C ABI declared in
include/gpufs_gb300.h with ctypes; there is no Python or CPU fallback, and
every entry point raises if the native library is missing.
"""
import ctypes
import os
import weakref

import numpy as np

# Enough hardware work queues that no host-worker stream shares one with the
# stream of a running file-system kernel (must be set before CUDA starts).
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

_HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(_HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libgpufs_gb300.so")

O_RDONLY = os.O_RDONLY
O_WRONLY = os.O_WRONLY
O_RDWR = os.O_RDWR
O_CREAT = os.O_CREAT
# reference flag names (libgpufs/fs_constants.h:86-90)
O_GRDONLY = O_RDONLY
O_GWRONLY = O_WRONLY
O_GCREAT = O_CREAT
O_GRDWR = O_RDWR
O_GWRONCE = O_CREAT | O_WRONLY

STAT_NAMES = ["hits", "misses", "evictions", "writebacks", "read_rpcs", "bytes_read_rpc", "opens", "closes",
              "timeouts", "errors", "conflict_evictions", "host_requests", "host_reads", "host_read_bytes",
              "host_writes", "host_write_bytes", "host_opens", "host_errors", "err_site", "rpc_submitted",
              "host_map_reads"]

ERR_TIMEOUT, ERR_IO, ERR_NOMEM, ERR_TABLE, ERR_ARG = 1, 2, 4, 8, 16
XXH64_NOALLOC_MAX_FILES = 1024  # GFS_XXH64_NOALLOC_MAX_FILES
CFG_NO_FILE_MAP = 1  # GFS_CFG_NO_FILE_MAP
CFG_RETAIN_CACHE = 2  # GFS_CFG_RETAIN_CACHE
CFG_HOST_TABLE = 4  # GFS_CFG_HOST_TABLE


class Config(ctypes.Structure):
    _fields_ = [("log_page", ctypes.c_uint32), ("max_files", ctypes.c_uint32), ("pool_bytes", ctypes.c_uint64),
                ("ring_slots", ctypes.c_uint32), ("host_workers", ctypes.c_uint32),
                ("staging_depth", ctypes.c_uint32), ("flags", ctypes.c_uint32), ("timeout_ns", ctypes.c_uint64),
                ("device", ctypes.c_int32), ("pad1", ctypes.c_uint32)]


_lib = None
_c_p = ctypes.c_void_p
_c_s = ctypes.c_char_p
_u64 = ctypes.c_uint64
_i64 = ctypes.c_longlong
_int = ctypes.c_int

_SIGS = {
    "gfs_default_config": (None, [ctypes.POINTER(Config)]),
    "gfs_create": (_int, [ctypes.POINTER(Config), ctypes.POINTER(_c_p)]),
    "gfs_destroy": (_int, [_c_p]),
    "gfs_run_handler": (_int, [_c_p, _int]),
    "gfs_kernel_stream": (_c_p, [_c_p]),
    "gfs_device_state": (_c_p, [_c_p]),
    "gfs_page_size": (ctypes.c_uint32, [_c_p]),
    "gfs_num_frames": (ctypes.c_uint32, [_c_p]),
    "gfs_pool_base": (_c_p, [_c_p]),
    "gfs_last_error": (ctypes.c_uint32, [_c_p, _int]),
    "gfs_get_stats": (_int, [_c_p, ctypes.POINTER(ctypes.c_ulonglong), _int]),
    "gfs_reset_stats": (_int, [_c_p]),
    "gfs_set_paused": (_int, [_c_p, _int]),
    "gfs_inject_read_errors": (_int, [_c_p, _int, _int]),
    "gfs_pread": (_i64, [_c_p, _c_s, _u64, _u64, _c_p, _int, _int]),
    "gfs_pread_dev": (_i64, [_c_p, _c_s, _u64, _u64, _c_p, _int, _int, ctypes.POINTER(ctypes.c_float)]),
    "gfs_pwrite": (_i64, [_c_p, _c_s, _int, _u64, _u64, _c_p, _int, _int]),
    "gfs_mmap_read": (_i64, [_c_p, _c_s, _u64, _u64, _c_p, _int, _int, _int]),
    "gfs_fstat_path": (_i64, [_c_p, _c_s]),
    "gfs_truncate_path": (_int, [_c_p, _c_s, _i64]),
    "gfs_unlink_path": (_int, [_c_p, _c_s]),
    "gfs_pwrite_fsync": (_i64, [_c_p, _c_s, _u64, _u64, _c_p]),
    "gfs_memcopy": (_int, [_c_p, _c_s, _c_s, _int, _int, _int, ctypes.POINTER(ctypes.c_float)]),
    "gfs_grep_open": (_int, [_c_p, _c_s, ctypes.POINTER(_c_s), _int, ctypes.POINTER(_c_p)]),
    "gfs_grep_run": (_int, [_c_p, _int, ctypes.POINTER(ctypes.c_float)]),
    "gfs_grep_run_direct": (_int, [_c_p, _int, ctypes.POINTER(ctypes.c_float)]),
    "gfs_grep_counts": (_int, [_c_p, _c_p]),
    "gfs_grep_device_counts": (_c_p, [_c_p]),
    "gfs_grep_info": (_int, [_c_p, ctypes.POINTER(ctypes.c_longlong), _int]),
    "gfs_grep_close": (_int, [_c_p]),
    "gfs_grep_text": (_int, [_c_p, _c_s, ctypes.POINTER(_c_s), _int, _c_p, _int]),
    "gfs_grep_batch": (_int, [_c_p, _int, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_float)]),
    "gfs_serve_open": (_int, [_c_p, _c_s, ctypes.POINTER(_c_s), _int, ctypes.POINTER(_c_s), _int,
                              ctypes.POINTER(_c_p)]),
    "gfs_serve_run": (_int, [_c_p, _c_p, _int, _c_p, _u64, _int]),
    "gfs_serve_close": (_int, [_c_p]),
    "gfs_serve_warps_per_sm": (_int, [_c_p, _int]),
    "gfs_serve_service_hist": (_int, [_c_p, _c_p, _int]),
    "gfs_grep_bench": (_int, [_c_p, _int, _int, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "gfs_drop_cache": (_i64, [_c_p]),
    "gfs_retained_pages": (_i64, [_c_p]),
    "gfs_release_retained": (_int, []),
    "gfs_bigmatrix": (_int, [_c_p, _c_s, _c_s, _c_s, _int, _int, ctypes.POINTER(ctypes.c_float)]),
    "gfs_bigmatrix_direct": (_int, [_c_p, _c_s, _c_s, _c_s, _int, _int, ctypes.POINTER(ctypes.c_float)]),
    "gfs_xxh64_files": (_int, [_c_p, ctypes.POINTER(_c_s), _int, ctypes.POINTER(ctypes.c_ulonglong),
                               ctypes.POINTER(ctypes.c_float)]),
    "gfs_xxh64_files_noalloc": (_int, [_c_p, ctypes.POINTER(_c_s), _int, ctypes.POINTER(ctypes.c_ulonglong)]),
    "gfs_measure_link": (_int, [_u64, _int, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "gfs_measure_cold_paths": (_int, [_c_s, _int, _u64, _int, ctypes.POINTER(ctypes.c_float), _int]),
    "gfs_cm_create": (_int, [_int, _int, ctypes.c_ulonglong, ctypes.POINTER(_c_p)]),
    "gfs_cm_destroy": (_int, [_c_p]),
    "gfs_cm_n_params": (_int, [_c_p]),
    "gfs_cm_get_params": (_int, [_c_p, _c_p]),
    "gfs_cm_set_params": (_int, [_c_p, _c_p]),
    "gfs_cm_set_data": (_int, [_c_p, _c_p, _c_p, _int]),
    "gfs_cm_grad": (_int, [_c_p, _c_p, ctypes.POINTER(ctypes.c_float)]),
    "gfs_cm_train": (_int, [_c_p, _int, ctypes.c_float, _c_p]),
    "gfs_cm_predict": (_int, [_c_p, _c_p, _int, _c_p]),
}


def lib():
    """Load libgpufs_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("gpufs_gb300: native library missing (%s); run gpufs_gb300.build.build()" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_GLOBAL)
    for name, (res, args) in _SIGS.items():
        if hasattr(L, name):
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
    _lib = L
    return L


def _p(path):
    b = os.fsencode(path)
    if len(b) >= 64:
        raise ValueError("path longer than 63 bytes (FILENAME_SIZE): %r" % path)
    return b


class GfsError(OSError):
    pass


def release_retained_cache():
    """Free a buffer cache that a closed Session(retain_cache=True) kept and
    no later session took over; True if one was freed."""
    return bool(lib().gfs_release_retained())


def _check(rc, what):
    if rc < 0:
        raise GfsError(-rc, "%s failed: %s" % (what, os.strerror(-rc) if -rc < 200 else str(rc)))
    return rc


class Session:
    """One file-system session on one GPU (initializer() .. delete GPUGlobals)."""

    def __init__(self, log_page=16, pool_bytes=2 << 30, max_files=1024, ring_slots=4096, host_workers=8,
                 staging_depth=8, timeout_s=30.0, device=0, file_map=True, retain_cache=False, host_table=False):
        """retain_cache: keep the buffer cache in HBM when the session closes,
        for the next session of this process with the same log_page,
        pool_bytes, max_files and device (kept only if every file is closed
        and every page clean); see retained_pages.  host_table: build grep
        dictionary tables on the host (the device build's fallback)."""
        L = lib()
        c = Config()
        L.gfs_default_config(ctypes.byref(c))
        c.log_page = log_page
        c.pool_bytes = pool_bytes
        c.max_files = max_files
        c.ring_slots = ring_slots
        c.host_workers = host_workers
        c.staging_depth = staging_depth
        c.flags = ((0 if file_map else CFG_NO_FILE_MAP) | (CFG_RETAIN_CACHE if retain_cache else 0) |
                   (CFG_HOST_TABLE if host_table else 0))
        c.timeout_ns = int(timeout_s * 1e9)
        c.device = device
        h = ctypes.c_void_p()
        _check(L.gfs_create(ctypes.byref(c), ctypes.byref(h)), "gfs_create")
        self._h = h
        self.L = L
        self._children = weakref.WeakSet()  # open Grep plans and Servers of this session
        self.page_size = L.gfs_page_size(h)
        self.n_frames = L.gfs_num_frames(h)
        # valid pages taken over from a cache an earlier session retained
        self.retained_pages = int(L.gfs_retained_pages(h))

    @property
    def handle(self):
        return self._h

    def close(self):
        """Close the session's open Grep plans and Servers (their files and
        device memory belong to it), then end the session."""
        if not self._h:
            return
        try:
            for ch in list(self._children):
                ch.close()
        finally:
            self._children.clear()
            self.L.gfs_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- device API driven from the host --
    def pread(self, path, off=0, size=None, nblocks=8, nthreads=256):
        if size is None:
            size = max(0, os.path.getsize(path) - off)
        out = np.empty(size, dtype=np.uint8)
        n = _check(self.L.gfs_pread(self._h, _p(path), off, size, out.ctypes.data if size else None, nblocks,
                                    nthreads), "gfs_pread")
        return out[:n]

    def pread_dev(self, path, off, size, dev_ptr, nblocks=8, nthreads=256):
        ms = ctypes.c_float(0)
        n = _check(self.L.gfs_pread_dev(self._h, _p(path), off, size, dev_ptr, nblocks, nthreads, ctypes.byref(ms)),
                   "gfs_pread_dev")
        return n, ms.value

    def pwrite(self, path, data, off=0, oflags=O_GWRONCE, nblocks=8, nthreads=256):
        a = np.ascontiguousarray(np.frombuffer(data, dtype=np.uint8) if not isinstance(data, np.ndarray) else
                                 data.view(np.uint8).ravel())
        return _check(self.L.gfs_pwrite(self._h, _p(path), oflags, off, a.size, a.ctypes.data if a.size else None,
                                        nblocks, nthreads), "gfs_pwrite")

    def pwrite_fsync(self, path, data, off=0):
        a = np.ascontiguousarray(np.frombuffer(data, dtype=np.uint8))
        return _check(self.L.gfs_pwrite_fsync(self._h, _p(path), off, a.size, a.ctypes.data), "gfs_pwrite_fsync")

    def mmap_read(self, path, off=0, size=None, nblocks=8, nthreads=256, warp_api=False):
        if size is None:
            size = max(0, os.path.getsize(path) - off)
        out = np.empty(size, dtype=np.uint8)
        n = _check(self.L.gfs_mmap_read(self._h, _p(path), off, size, out.ctypes.data if size else None, nblocks,
                                        nthreads, 1 if warp_api else 0), "gfs_mmap_read")
        return out[:n]

    def fstat(self, path):
        return _check(self.L.gfs_fstat_path(self._h, _p(path)), "gfs_fstat_path")

    def truncate(self, path, size):
        return _check(self.L.gfs_truncate_path(self._h, _p(path), size), "gfs_truncate_path")

    def unlink(self, path):
        return _check(self.L.gfs_unlink_path(self._h, _p(path)), "gfs_unlink_path")

    def memcopy(self, src, dst, nblocks=112, nthreads=256, mode=0):
        ms = ctypes.c_float(0)
        _check(self.L.gfs_memcopy(self._h, _p(src), _p(dst), nblocks, nthreads, mode, ctypes.byref(ms)),
               "gfs_memcopy")
        return ms.value

    def bigmatrix(self, vec_path, mat_path, out_path, nblocks=152, nthreads=256, direct=False):
        """y = A x through gmmap (samples/bigmatrix_mmap); returns kernel ms.
        direct=True reads the matrix straight from its host mapping (one pass
        over a cold matrix)."""
        ms = ctypes.c_float(0)
        fn = self.L.gfs_bigmatrix_direct if direct else self.L.gfs_bigmatrix
        _check(fn(self._h, _p(vec_path), _p(mat_path), _p(out_path), nblocks, nthreads, ctypes.byref(ms)),
               "gfs_bigmatrix")
        return ms.value

    def xxh64_files(self, paths):
        """XXH64 (seed 0) of each file, read through the buffer cache."""
        out = (ctypes.c_ulonglong * len(paths))()
        ms = ctypes.c_float(0)
        _check(self.L.gfs_xxh64_files(self._h, _paths(paths), len(paths), out, ctypes.byref(ms)),
               "gfs_xxh64_files")
        return [int(v) for v in out], ms.value

    def xxh64_files_noalloc(self, paths):
        """gfs_xxh64_files without any allocation (at most XXH64_NOALLOC_MAX_FILES
        files; calls on one device must not overlap)."""
        out = (ctypes.c_ulonglong * max(len(paths), 1))()
        _check(self.L.gfs_xxh64_files_noalloc(self._h, _paths(paths), len(paths), out),
               "gfs_xxh64_files_noalloc")
        return [int(v) for v in out[:len(paths)]]

    # -- introspection / fault injection --
    def stats(self):
        arr = (ctypes.c_ulonglong * len(STAT_NAMES))()
        n = self.L.gfs_get_stats(self._h, arr, len(STAT_NAMES))
        return {STAT_NAMES[i]: int(arr[i]) for i in range(n)}

    def reset_stats(self):
        self.L.gfs_reset_stats(self._h)

    def error_report(self):
        st = self.stats()
        return "error bits 0x%x, first failure site %d errno %d, stats %s" % (
            self.last_error(clear=False), st.get("err_site", 0) >> 16, st.get("err_site", 0) & 0xFFFF, st)

    def last_error(self, clear=True):
        return int(self.L.gfs_last_error(self._h, 1 if clear else 0))

    def drop_cache(self):
        return _check(self.L.gfs_drop_cache(self._h), "gfs_drop_cache")

    def set_paused(self, paused):
        self.L.gfs_set_paused(self._h, 1 if paused else 0)

    def inject_read_errors(self, count, err=5):
        self.L.gfs_inject_read_errors(self._h, count, err)


def _paths(paths):
    arr = (ctypes.c_char_p * len(paths))(*[_p(x) for x in paths])
    return arr


class Grep:
    """grep_text plan: dictionary table on the device, corpus files open in
    the session (samples/grep_text/grep_text_gpu.cu:193-387)."""

    def __init__(self, sess, dict_path, paths):
        self.s = sess
        self.paths = list(paths)
        h = ctypes.c_void_p()
        _check(sess.L.gfs_grep_open(sess.handle, _p(dict_path), _paths(self.paths), len(self.paths),
                                    ctypes.byref(h)), "gfs_grep_open")
        self._h = h
        sess._children.add(self)
        self._info()

    def _info(self):
        info = (ctypes.c_longlong * 10)()
        self.s.L.gfs_grep_info(self._h, info, 10)
        (self.n_words, self.n_files, self.slots, self.smem_table, self.smem_bytes, self.chunks, self.status,
         self.status_site, self.build_us, self.open_us) = [int(v) for v in info]

    def run(self, n_ctas=0, direct=False):
        """One scan; direct=True reads files with a registered host mapping
        straight from it, bypassing the buffer cache."""
        ms = ctypes.c_float(0)
        fn = self.s.L.gfs_grep_run_direct if direct else self.s.L.gfs_grep_run
        rc = fn(self._h, n_ctas, ctypes.byref(ms))
        if rc < 0:
            self._info()
            raise GfsError(-rc, "gfs_grep_run failed: status 0x%x site 0x%x, session %s" % (
                self.status, self.status_site, self.s.error_report()))
        return ms.value

    def batch(self, n_ctas=0):
        """Batched form: counts and per-file XXH64 in one persistent graph
        launch; returns (xxh64 list, kernel ms).  counts() then holds the
        counts."""
        out = (ctypes.c_ulonglong * max(self.n_files, 1))()
        ms = ctypes.c_float(0)
        rc = self.s.L.gfs_grep_batch(self._h, n_ctas, out, ctypes.byref(ms))
        if rc < 0:
            self._info()
            raise GfsError(-rc, "gfs_grep_batch failed: status 0x%x site 0x%x, session %s" % (
                self.status, self.status_site, self.s.error_report()))
        return [int(v) for v in out[:self.n_files]], ms.value

    def counts(self):
        out = np.zeros((self.n_words, self.n_files), dtype=np.uint32)
        _check(self.s.L.gfs_grep_counts(self._h, out.ctypes.data), "gfs_grep_counts")
        return out

    def bench(self, steps, n_ctas=0):
        """(total_ms, mean scan-kernel ms) of `steps` back-to-back runs."""
        tot = ctypes.c_float(0)
        scan = ctypes.c_float(0)
        _check(self.s.L.gfs_grep_bench(self._h, n_ctas, steps, ctypes.byref(tot), ctypes.byref(scan)),
               "gfs_grep_bench")
        return tot.value, scan.value

    def device_counts(self):
        return self.s.L.gfs_grep_device_counts(self._h)

    def close(self):
        if self._h:
            h, self._h = self._h, None
            self.s._children.discard(self)
            if self.s.handle:  # after the session has ended there is nothing left to close
                _check(self.s.L.gfs_grep_close(h), "gfs_grep_close")

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def grep_text(sess, dict_path, paths, n_ctas=0):
    """One call: open + scan + counts + close; returns counts[word, file]."""
    n_words = os.path.getsize(dict_path) // 32
    out = np.zeros((n_words, len(paths)), dtype=np.uint32)
    _check(sess.L.gfs_grep_text(sess.handle, _p(dict_path), _paths(paths), len(paths),
                                out.ctypes.data if out.size else None, n_ctas), "gfs_grep_text")
    return out


def measure_cold_paths(path, streams=16, chunk=2 << 20, reps=3):
    """Cold-read ceilings for one file (GB/s): pinned single copy, pinned
    chunked over streams, registered file mapping chunked over streams, a
    kernel reading pinned memory, a kernel reading the file mapping."""
    out = (ctypes.c_float * 7)()
    _check(lib().gfs_measure_cold_paths(os.fsencode(path), streams, chunk, reps, out, 7), "gfs_measure_cold_paths")
    keys = ("pinned_1_copy", "pinned_streams", "file_map_streams", "kernel_pinned", "kernel_file_map",
            "kernel_file_map_slices", "kernel_file_map_slices_1warp")
    return dict(zip(keys, [float(v) for v in out]))


def measure_link(nbytes=1 << 30, reps=5):
    """Pinned host->device and device->host copy bandwidth in GB/s."""
    a = ctypes.c_float(0)
    b = ctypes.c_float(0)
    _check(lib().gfs_measure_link(nbytes, reps, ctypes.byref(a), ctypes.byref(b)), "gfs_measure_link")
    return a.value, b.value


# ---- served form ----
SV_READ, SV_GREP, SV_WRITE = 1, 2, 3
SERVE_REQ = np.dtype([("op", "<u4"), ("file", "<u4"), ("offset", "<u8"), ("length", "<u8"), ("arrival_ns", "<u8")])
SERVE_RES = np.dtype([("result", "<u8"), ("status", "<i4"), ("pad", "<u4"), ("submit_ns", "<u8"),
                      ("complete_ns", "<u8")])


class Server:
    """Served form: a persistent device loop over a request ring; files stay
    open on the device for the server's life."""

    def __init__(self, sess, dict_path, paths, out_paths=()):
        self.s = sess
        self.paths = list(paths)
        self.out_paths = list(out_paths)
        h = ctypes.c_void_p()
        outs = _paths(self.out_paths) if self.out_paths else None
        _check(sess.L.gfs_serve_open(sess.handle, _p(dict_path), _paths(self.paths), len(self.paths), outs,
                                     len(self.out_paths), ctypes.byref(h)), "gfs_serve_open")
        self._h = h
        sess._children.add(self)

    def run(self, reqs, inflight_pages=1 << 62, warps_per_sm=8):
        """reqs: SERVE_REQ array sorted by arrival_ns.  Returns a SERVE_RES array."""
        reqs = np.ascontiguousarray(reqs, dtype=SERVE_REQ)
        res = np.zeros(reqs.size, dtype=SERVE_RES)
        _check(self.s.L.gfs_serve_run(self._h, reqs.ctypes.data if reqs.size else None, reqs.size,
                                      res.ctypes.data if reqs.size else None, int(inflight_pages), warps_per_sm),
               "gfs_serve_run")
        return res

    def service_hist(self):
        """The last run's device-side histogram of service times: element b
        counts requests served in [2**b, 2**(b+1)) ns."""
        out = np.zeros(64, dtype=np.uint64)
        _check(self.s.L.gfs_serve_service_hist(self._h, out.ctypes.data, out.size), "gfs_serve_service_hist")
        return out

    def warps_per_sm(self, asked=32):
        """Serving warps per SM a run asked for `asked` uses (whole blocks of
        8, capped at what the device holds at once)."""
        return _check(self.s.L.gfs_serve_warps_per_sm(self._h, asked), "gfs_serve_warps_per_sm")

    def close(self):
        if self._h:
            h, self._h = self._h, None
            self.s._children.discard(self)
            if self.s.handle:  # after the session has ended there is nothing left to close
                _check(self.s.L.gfs_serve_close(h), "gfs_serve_close")

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def serve_pattern(offset, length, req_id):
    """The bytes a GFS_SV_WRITE request writes (the device's pattern)."""
    x = np.arange(offset, offset + length, dtype=np.uint64).astype(np.uint32)
    v = (x * np.uint32(0x9E3779B1) + np.uint32((req_id * 0x85EBCA77) & 0xFFFFFFFF)) >> np.uint32(24)
    return v.astype(np.uint8)

"""Cross-session buffer cache (GFS_CFG_RETAIN_CACHE): pages a session read
are found by the next session of the process with the same geometry,
without host reads; a file changed on the host in between is read again
(the reopen check of libgpufs/fs_calls.cu:197-218, across sessions); any
other geometry, or a session without the flag, starts empty."""
import os
import time

import numpy as np
import pytest

import gpufs_gb300 as g
from gpufs_gb300 import datagen
from oracle import oracle

pytestmark = pytest.mark.gpu

GEOM = dict(log_page=16, pool_bytes=64 << 20, max_files=64, timeout_s=20)


def _mk(path, n, seed):
    a = np.random.default_rng(seed).integers(0, 256, n, dtype=np.uint8)
    a.tofile(path)
    return a


@pytest.fixture(autouse=True)
def _nothing_kept(built):
    g.release_retained_cache()
    yield
    g.release_retained_cache()


def test_pages_survive_into_the_next_session(shm_dir):
    p = os.path.join(shm_dir, "r.bin")
    a = _mk(p, (4 << 20) + 1000, seed=1)
    with g.Session(retain_cache=True, **GEOM) as s:
        assert s.retained_pages == 0
        assert np.array_equal(s.pread(p), a)
        assert s.stats()["misses"] >= 65
    with g.Session(retain_cache=True, **GEOM) as s:
        assert s.retained_pages == 65  # 4 MiB + 1000 B in 64 KiB pages
        s.reset_stats()
        assert np.array_equal(s.pread(p), a)
        st = s.stats()
        assert st["misses"] == 0 and st["host_reads"] == 0 and st["hits"] >= 65
        assert s.last_error() == 0


def test_changed_file_is_read_again(shm_dir):
    p = os.path.join(shm_dir, "c.bin")
    a = _mk(p, 1 << 20, seed=2)
    with g.Session(retain_cache=True, **GEOM) as s:
        assert np.array_equal(s.pread(p), a)
    time.sleep(0.01)
    b = _mk(p, 1 << 20, seed=3)  # same size and inode, new ctime
    with g.Session(retain_cache=True, **GEOM) as s:
        assert s.retained_pages == 16
        s.reset_stats()
        assert np.array_equal(s.pread(p), b)
        assert s.stats()["misses"] >= 16
        assert s.last_error() == 0


def test_other_geometry_or_plain_session_starts_empty(shm_dir):
    p = os.path.join(shm_dir, "o.bin")
    a = _mk(p, 1 << 20, seed=4)
    other = dict(GEOM, pool_bytes=32 << 20)
    with g.Session(retain_cache=True, **GEOM) as s:
        s.pread(p)
    with g.Session(retain_cache=True, **other) as s:  # another pool size: the kept cache is freed
        assert s.retained_pages == 0
        assert np.array_equal(s.pread(p), a)
    with g.Session(**GEOM) as s:  # no flag: frees the cache kept above and keeps none
        assert s.retained_pages == 0
    assert not g.release_retained_cache()
    with g.Session(retain_cache=True, **GEOM) as s:
        s.pread(p)
    assert g.release_retained_cache()
    with g.Session(retain_cache=True, **GEOM) as s:
        assert s.retained_pages == 0
        assert np.array_equal(s.pread(p), a)


def test_grep_corpus_stays_resident_across_sessions(shm_dir):
    paths, dpath = datagen.grep_corpus(shm_dir, n_files=3, total_bytes=3 * (1 << 20) + 555, n_vocab=2000,
                                       n_dict=500, seed=5)
    with g.Session(retain_cache=True, **GEOM) as s:
        with g.Grep(s, dpath, paths) as gr:
            gr.run()
            first = gr.counts()
    with g.Session(retain_cache=True, **GEOM) as s:
        assert s.retained_pages >= 48
        s.reset_stats()
        with g.Grep(s, dpath, paths) as gr:
            gr.run()
            second = gr.counts()
        assert s.stats()["misses"] == 0
        assert s.last_error() == 0
    want = oracle.grep_counts(open(dpath, "rb").read(), [open(q, "rb").read() for q in paths], mode="fast")
    assert np.array_equal(first, want)
    assert np.array_equal(second, want)


_RESET_SCRIPT = r"""
import ctypes, os, sys
sys.path.insert(0, %r)
import numpy as np
import gpufs_gb300 as g
p = %r
a = np.random.default_rng(7).integers(0, 256, (1 << 20) + 33, dtype=np.uint8)
a.tofile(p)
geom = dict(log_page=16, pool_bytes=64 << 20, max_files=64, timeout_s=20)
rt = ctypes.CDLL("libcudart.so.13")
with g.Session(retain_cache=True, **geom) as s:
    assert np.array_equal(s.pread(p), a)
assert rt.cudaDeviceReset() == 0
# the kept cache did not survive the reset: a new session starts empty, and
# reads the file again
with g.Session(retain_cache=True, **geom) as s:
    assert s.retained_pages == 0, s.retained_pages
    assert np.array_equal(s.pread(p), a)
    assert s.last_error() == 0
# a cache kept and then orphaned by a reset is dropped (not freed) on release
with g.Session(retain_cache=True, **geom) as s:
    assert np.array_equal(s.pread(p), a)
assert rt.cudaDeviceReset() == 0
assert g.release_retained_cache() == 1
with g.Session(**geom) as s:
    assert np.array_equal(s.pread(p), a)
print("reset-guard-ok")
"""


def test_kept_cache_does_not_survive_a_device_reset(shm_dir):
    """A cudaDeviceReset between sessions frees a kept cache's memory under
    it: the next retaining session must not take it over (its pointers are
    checked, and a token in device memory read back, before any use), and
    releasing such a cache frees nothing that is no longer ours.  Runs in a
    child process, since the reset ends every CUDA object of the process."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = _RESET_SCRIPT % (root, os.path.join(shm_dir, "reset.bin"))
    out = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and "reset-guard-ok" in out.stdout, out.stdout[-2000:] + out.stderr[-2000:]

"""gfs_xxh64_files_noalloc: the allocation-free XXH64 entry point.

Its scratch is a fixed file-scope device array, so this file is collected
last (it must pass alone and after every other test) and compares the
entry point with gfs_xxh64_files on two calls in a row, against the oracle.
"""
import errno
import os

import numpy as np
import pytest

import gpufs_gb300 as g
from gpufs_gb300 import datagen
from oracle import oracle

pytestmark = pytest.mark.gpu


def _files(d, n, seed):
    rng = np.random.default_rng(seed)
    paths = []
    for i in range(n):
        p = os.path.join(d, "na%04d_%d.bin" % (i, seed))
        size = int(rng.choice([0, 1, 31, 32, 4095, 65536 + 7, 300001, 1 << 20]))
        datagen.uniform_bytes(p, size, seed=seed * 1000 + i)
        paths.append(p)
    return paths


def test_noalloc_matches_allocating_entry_point(built, shm_dir):
    a = _files(shm_dir, 70, seed=1)
    b = _files(shm_dir, 9, seed=2)
    with g.Session(log_page=16, pool_bytes=64 << 20, max_files=256, timeout_s=20) as s:
        for paths in (a, b):
            want = [oracle.xxh64(np.fromfile(p, dtype=np.uint8)) for p in paths]
            ref, _ = s.xxh64_files(paths)
            first = s.xxh64_files_noalloc(paths)
            second = s.xxh64_files_noalloc(paths)
            assert ref == want
            assert first == ref
            assert second == ref
        assert s.last_error() == 0


def test_noalloc_limit_is_an_error(built, shm_dir):
    p = _files(shm_dir, 1, seed=3)[0]
    with g.Session(log_page=16, pool_bytes=16 << 20, timeout_s=20) as s:
        with pytest.raises(g.GfsError) as ei:
            s.xxh64_files_noalloc([p] * (g.XXH64_NOALLOC_MAX_FILES + 1))
        assert ei.value.errno == errno.E2BIG
        # the limit itself is accepted, and the session stays usable
        h = s.xxh64_files_noalloc([p] * g.XXH64_NOALLOC_MAX_FILES)
        assert len(set(h)) == 1 and h[0] == oracle.xxh64(np.fromfile(p, dtype=np.uint8))

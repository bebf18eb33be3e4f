"""bigmatrix_mmap and per-file XXH64 through the GPU file system, against
the oracle (FP64 host GEMV; XXH64 from the public specification)."""
import os

import numpy as np
import pytest

import gpufs_gb300 as g
from gpufs_gb300 import datagen
from oracle import oracle

pytestmark = pytest.mark.gpu


# (300, 65536, 21), (200, 1024, 16) and (2048, 2048, 16) take the lookahead
# form (every group of eight rows inside one page; two groups per page in the
# second; the third through a pool smaller than the matrix); the others go
# row by row where rows cross pages
@pytest.mark.parametrize("rows,cols,log_page,pool_mb", [(512, 4096, 16, 256), (300, 65536, 21, 256), (97, 1000, 12, 256),
                                                        (64, 70000, 16, 256), (200, 1024, 16, 256),
                                                        (2048, 2048, 16, 8)])
def test_bigmatrix_matches_fp64(built, shm_dir, rows, cols, log_page, pool_mb):
    vp, mp, op = (os.path.join(shm_dir, n) for n in ("v.f32", "m.f32", "o.f32"))
    datagen.normal_f32(vp, cols, seed=3)
    datagen.normal_f32(mp, rows * cols, seed=4)
    with open(op, "wb") as f:
        f.write(b"\xff" * 1000)  # stale bytes: the sample truncates its output first
    with g.Session(log_page=log_page, pool_bytes=pool_mb << 20, timeout_s=20) as s:
        s.bigmatrix(vp, mp, op, nblocks=37, nthreads=256)
        assert s.last_error() == 0, s.error_report()
        if pool_mb * (1 << 20) < rows * cols * 4:
            assert s.stats()["evictions"] > 0
    A = np.fromfile(mp, dtype=np.float32).reshape(rows, cols)
    x = np.fromfile(vp, dtype=np.float32)
    y = np.fromfile(op, dtype=np.float32)
    assert y.size == rows
    y64, ay = oracle.gemv_f64(A, x)
    # norm-wise and per-element (relative to sum |a_ij x_j|) within 1e-5
    assert np.linalg.norm(y - y64) / np.linalg.norm(y64) <= 1e-5
    assert np.all(np.abs(y - y64) <= 1e-5 * ay)


@pytest.mark.parametrize("rows,cols", [(96, 65536), (37, 8192 + 4), (11, 1023)])
def test_bigmatrix_direct_matches_fp64(built, shm_dir, rows, cols):
    """The one-pass form reads the matrix straight from its host mapping (or
    through the cache when it has none) within the same bounds."""
    vp, mp, op = (os.path.join(shm_dir, n) for n in ("v.f32", "m.f32", "o.f32"))
    datagen.normal_f32(vp, cols, seed=7)
    datagen.normal_f32(mp, rows * cols, seed=8)
    with g.Session(log_page=16, pool_bytes=256 << 20, timeout_s=20) as s:
        s.reset_stats()
        s.bigmatrix(vp, mp, op, nblocks=7, nthreads=256, direct=True)
        assert s.last_error() == 0, s.error_report()
        mat_pages = (rows * cols * 4 + 65535) // 65536
        if rows * cols * 4 >= 65536:  # mapped: the matrix never enters the cache
            assert s.stats()["misses"] < mat_pages
    A = np.fromfile(mp, dtype=np.float32).reshape(rows, cols)
    x = np.fromfile(vp, dtype=np.float32)
    y = np.fromfile(op, dtype=np.float32)
    assert y.size == rows
    y64, ay = oracle.gemv_f64(A, x)
    assert np.linalg.norm(y - y64) / np.linalg.norm(y64) <= 1e-5
    assert np.all(np.abs(y - y64) <= 1e-5 * ay)


def test_bigmatrix_deterministic(built, shm_dir):
    vp, mp = os.path.join(shm_dir, "v.f32"), os.path.join(shm_dir, "m.f32")
    datagen.normal_f32(vp, 8192, seed=5)
    datagen.normal_f32(mp, 256 * 8192, seed=6)
    outs = []
    with g.Session(log_page=16, pool_bytes=64 << 20, timeout_s=20) as s:
        for i in range(2):
            op = os.path.join(shm_dir, "o%d.f32" % i)
            s.bigmatrix(vp, mp, op, nblocks=19, nthreads=128)
            outs.append(open(op, "rb").read())
    assert outs[0] == outs[1]


def test_xxh64_files(built, shm_dir):
    sizes = [0, 1, 7, 31, 32, 33, 100, 4095, 4096, 65537, 1 << 20, 3 * (1 << 20) + 17]
    paths = []
    for i, n in enumerate(sizes):
        p = os.path.join(shm_dir, "x%02d.bin" % i)
        datagen.uniform_bytes(p, n, seed=40 + i)
        paths.append(p)
    for lp in (12, 16):
        with g.Session(log_page=lp, pool_bytes=64 << 20, timeout_s=20) as s:
            got, _ = s.xxh64_files(paths)
            want = oracle.xxh64_many([np.fromfile(p, dtype=np.uint8) for p in paths])
            assert got == want
            assert s.last_error() == 0

"""Parity of the GPU file system with the host file, through the C ABI.

Every byte read through gread/gmmap must equal the host file; every byte
written through gwrite must land in the host file (write-once pages OR-merged
as the reference's diff_and_merge does); failures come back as errors, never
as a hang or a fault.
"""
import errno
import os
import time

import numpy as np
import pytest

import gpufs_gb300 as g
from gpufs_gb300 import datagen
from oracle import oracle

pytestmark = pytest.mark.gpu


def _mk(path, n, seed=1):
    datagen.uniform_bytes(path, n, seed=seed)
    return np.fromfile(path, dtype=np.uint8)


@pytest.fixture(scope="module")
def sess(built):
    s = g.Session(log_page=16, pool_bytes=256 << 20, max_files=256, timeout_s=20)
    yield s
    s.close()


def test_pread_whole_and_slices(sess, shm_dir):
    p = os.path.join(shm_dir, "a.bin")
    want = _mk(p, 5 * (1 << 20) + 777)
    got = sess.pread(p, 0, want.size, nblocks=8)
    assert np.array_equal(got, want)
    rng = np.random.default_rng(5)
    for _ in range(12):
        off = int(rng.integers(0, want.size))
        n = int(rng.integers(0, 300000))
        got = sess.pread(p, off, n, nblocks=int(rng.integers(1, 9)), nthreads=int(rng.choice([32, 96, 256, 1024])))
        assert np.array_equal(got, want[off:off + n]), (off, n)
    # end of file clamps; past the end reads nothing
    assert np.array_equal(sess.pread(p, want.size - 10, 1000, nblocks=1), want[-10:])
    assert sess.pread(p, want.size + 5, 100, nblocks=1).size == 0
    assert sess.last_error() == 0


def test_empty_and_tiny_files(sess, shm_dir):
    e = os.path.join(shm_dir, "empty.bin")
    open(e, "wb").close()
    assert sess.pread(e, 0, 100, nblocks=2).size == 0
    t = os.path.join(shm_dir, "tiny.bin")
    open(t, "wb").write(b"xyz")
    assert bytes(sess.pread(t, 0, 3, nblocks=1)) == b"xyz"
    assert sess.fstat(t) == 3


@pytest.mark.parametrize("log_page", [12, 16, 21])
def test_page_sizes(built, shm_dir, log_page):
    p = os.path.join(shm_dir, "b.bin")
    want = _mk(p, 9 * (1 << 20) + 4097, seed=3)
    with g.Session(log_page=log_page, pool_bytes=64 << 20, timeout_s=20) as s:
        got = s.pread(p, 0, want.size, nblocks=16)
        assert np.array_equal(got, want)
        got = s.mmap_read(p, 123, 3 << 20, nblocks=4)
        assert np.array_equal(got, want[123:123 + (3 << 20)])
        assert s.last_error() == 0


def test_second_read_hits_cache(sess, shm_dir):
    p = os.path.join(shm_dir, "c.bin")
    want = _mk(p, 8 << 20, seed=4)
    sess.reset_stats()
    assert np.array_equal(sess.pread(p, 0, want.size, nblocks=8), want)
    st1 = sess.stats()
    assert st1["misses"] == (8 << 20) // sess.page_size
    # the misses were filled by the reading blocks from the file's mapping
    assert st1["read_rpcs"] == 0 and st1["host_read_bytes"] == 0
    sess.reset_stats()
    assert np.array_equal(sess.pread(p, 0, want.size, nblocks=8), want)
    st2 = sess.stats()
    assert st2["misses"] == 0 and st2["host_reads"] == 0


def test_mmap_block_and_warp(sess, shm_dir):
    p = os.path.join(shm_dir, "m.bin")
    want = _mk(p, 3 * (1 << 20) + 5, seed=6)
    for warp in (False, True):
        got = sess.mmap_read(p, 0, want.size, nblocks=6, nthreads=128, warp_api=warp)
        assert np.array_equal(got, want)
        got = sess.mmap_read(p, 70001, 500000, nblocks=3, nthreads=64, warp_api=warp)
        assert np.array_equal(got, want[70001:570001])


def test_pwrite_new_file(sess, shm_dir):
    p = os.path.join(shm_dir, "w.bin")
    rng = np.random.default_rng(7)
    data = rng.integers(0, 256, 3 * (1 << 20) + 999, dtype=np.uint8)
    assert sess.pwrite(p, data, 0, g.O_GWRONCE, nblocks=8) == data.size
    got = np.fromfile(p, dtype=np.uint8)
    assert np.array_equal(got, data)
    # and reading it back through the file system
    assert np.array_equal(sess.pread(p, 0, data.size, nblocks=4), data)


def test_pwrite_partial_pages_rdwr(sess, shm_dir):
    p = os.path.join(shm_dir, "rw.bin")
    base = _mk(p, (1 << 20) + 100, seed=8)
    rng = np.random.default_rng(9)
    exp = base.copy()
    for _ in range(5):
        off = int(rng.integers(0, base.size - 1000))
        n = int(rng.integers(1, 200000))
        d = rng.integers(0, 256, n, dtype=np.uint8)
        sess.pwrite(p, d, off, g.O_GRDWR, nblocks=int(rng.integers(1, 5)))
        end = off + n
        if end > exp.size:
            exp = np.concatenate([exp, np.zeros(end - exp.size, np.uint8)])
        exp[off:end] = d
        got = np.fromfile(p, dtype=np.uint8)
        assert np.array_equal(got, exp), (off, n)


def test_write_once_or_merge(sess, shm_dir):
    """O_GWRONCE pages are never read; at write-back they are OR-ed into the
    existing bytes (host_loop.h:76-137), so unwritten bytes keep old content."""
    p = os.path.join(shm_dir, "once.bin")
    old = _mk(p, 200000, seed=10)
    d = np.full(1000, 0x0F, np.uint8)
    off = 70000
    sess.pwrite(p, d, off, g.O_GWRONCE, nblocks=1)
    got = np.fromfile(p, dtype=np.uint8)
    exp = old.copy()
    exp[off:off + 1000] |= d
    assert np.array_equal(got, exp)


def test_memcopy_both_modes(sess, shm_dir):
    src = os.path.join(shm_dir, "src.bin")
    want = _mk(src, 7 * (1 << 20) + 12345, seed=11)
    for mode in (0, 1):
        dst = os.path.join(shm_dir, "dst%d.bin" % mode)
        sess.memcopy(src, dst, nblocks=112, nthreads=256, mode=mode)
        got = np.fromfile(dst, dtype=np.uint8)
        assert got.size == want.size
        assert oracle.xxh64(got) == oracle.xxh64(want)
    assert sess.last_error() == 0


def test_eviction_small_pool(built, shm_dir):
    p = os.path.join(shm_dir, "big.bin")
    want = _mk(p, 24 << 20, seed=12)
    with g.Session(log_page=16, pool_bytes=4 << 20, timeout_s=20) as s:
        for _ in range(2):
            assert np.array_equal(s.pread(p, 0, want.size, nblocks=4, nthreads=256), want)
        st = s.stats()
        assert st["evictions"] > 0
        assert s.last_error() == 0


def test_dirty_eviction_writes_back(built, shm_dir):
    p = os.path.join(shm_dir, "dirty.bin")
    rng = np.random.default_rng(13)
    data = rng.integers(0, 256, 12 << 20, dtype=np.uint8)
    with g.Session(log_page=16, pool_bytes=4 << 20, timeout_s=20) as s:
        s.pwrite(p, data, 0, g.O_GWRONCE, nblocks=2)
        st = s.stats()
        assert st["writebacks"] >= (12 << 20) // s.page_size
        assert s.last_error(clear=False) == 0, s.error_report()
    assert np.array_equal(np.fromfile(p, dtype=np.uint8), data)


def test_reopen_sees_host_change(sess, shm_dir):
    p = os.path.join(shm_dir, "chg.bin")
    a = _mk(p, 1 << 20, seed=14)
    assert np.array_equal(sess.pread(p, 0, a.size, nblocks=2), a)
    time.sleep(0.01)
    b = _mk(p, 1 << 20, seed=15)
    assert np.array_equal(sess.pread(p, 0, b.size, nblocks=2), b)


def test_fstat_truncate_unlink(sess, shm_dir):
    p = os.path.join(shm_dir, "t.bin")
    _mk(p, 300000, seed=16)
    assert sess.fstat(p) == 300000
    sess.truncate(p, 0)
    assert os.path.getsize(p) == 0
    assert sess.fstat(p) == 0
    sess.unlink(p)
    assert not os.path.exists(p)


def test_fsync_path(sess, shm_dir):
    p = os.path.join(shm_dir, "fs.bin")
    base = _mk(p, 100000, seed=17)
    d = np.arange(5000, dtype=np.uint8)
    sess.pwrite_fsync(p, d, 1234)
    base[1234:6234] = d
    assert np.array_equal(np.fromfile(p, dtype=np.uint8), base)


def test_missing_file_is_an_error(sess, shm_dir):
    with pytest.raises(g.GfsError) as ei:
        sess.pread(os.path.join(shm_dir, "nope.bin"), 0, 10, nblocks=1)
    assert ei.value.errno == errno.ENOENT
    sess.last_error()


def test_many_files_recycle_slots(built, shm_dir):
    with g.Session(log_page=12, pool_bytes=16 << 20, max_files=64, timeout_s=20) as s:
        for i in range(200):
            p = os.path.join(shm_dir, "f%03d" % i)
            w = _mk(p, 5000 + i, seed=100 + i)
            assert np.array_equal(s.pread(p, 0, w.size, nblocks=1, nthreads=64), w)
        assert s.last_error() == 0


def test_injected_read_error_propagates(built, shm_dir):
    p = os.path.join(shm_dir, "inj.bin")
    want = _mk(p, 1 << 20, seed=18)
    # without file mappings every miss is a host read, which the fault hits
    with g.Session(log_page=16, pool_bytes=16 << 20, timeout_s=20, file_map=False) as s:
        s.inject_read_errors(1, errno.EIO)
        with pytest.raises(g.GfsError) as ei:
            s.pread(p, 0, want.size, nblocks=1)
        assert ei.value.errno == errno.EIO
        assert s.last_error() & g.ERR_IO
        assert np.array_equal(s.pread(p, 0, want.size, nblocks=1), want)


def test_stalled_host_times_out(built, shm_dir):
    """A stalled host service is a bounded wait on the GPU: the call fails
    with ETIMEDOUT and the sticky timeout bit, and the GPU stays usable."""
    p = os.path.join(shm_dir, "stall.bin")
    _mk(p, 1 << 20, seed=19)
    with g.Session(log_page=16, pool_bytes=16 << 20, timeout_s=0.5) as s:
        s.set_paused(True)
        t0 = time.time()
        with pytest.raises(g.GfsError) as ei:
            s.pread(p, 0, 1 << 20, nblocks=2)
        assert ei.value.errno == errno.ETIMEDOUT
        assert time.time() - t0 < 30
        assert s.last_error() & g.ERR_TIMEOUT
    # a fresh session works
    with g.Session(log_page=16, pool_bytes=16 << 20, timeout_s=20) as s:
        w = np.fromfile(p, dtype=np.uint8)
        assert np.array_equal(s.pread(p, 0, w.size, nblocks=2), w)


def test_reads_use_registered_file_mapping(built, shm_dir):
    """Read-only opens get a registered mapping of the host file: gread's
    misses are filled by the reading block itself, with SM loads from the
    mapping (no request to the host at all), and so are gmmap's misses, by
    the mapping block or warp; a rewritten file (new size/ctime) is mapped
    afresh; with the mapping off every miss goes through pread into
    staging."""
    p = os.path.join(shm_dir, "mapped.bin")
    want = _mk(p, 3 * (1 << 20) + 5, seed=20)
    with g.Session(log_page=16, pool_bytes=64 << 20, timeout_s=20) as s:
        s.reset_stats()
        assert np.array_equal(s.pread(p, 0, want.size, nblocks=4), want)
        st = s.stats()
        assert st["misses"] == (want.size + 65535) // 65536
        assert st["read_rpcs"] == 0 and st["host_reads"] == 0
        # gmmap (block-collective, then warp-collective): the mapping
        # block or warp copies each missed page from the file's mapping
        for warp_api in (False, True):
            s.drop_cache()
            s.reset_stats()
            assert np.array_equal(s.mmap_read(p, 0, want.size, nblocks=4, warp_api=warp_api), want)
            st = s.stats()
            assert st["misses"] == (want.size + 65535) // 65536
            assert st["read_rpcs"] == 0 and st["host_reads"] == 0
        time.sleep(0.01)
        want2 = _mk(p, 2 * (1 << 20) + 77, seed=21)
        assert np.array_equal(s.pread(p, 0, want2.size, nblocks=3), want2)
        assert s.last_error() == 0
    with g.Session(log_page=16, pool_bytes=64 << 20, timeout_s=20, file_map=False) as s:
        s.reset_stats()
        assert np.array_equal(s.pread(p, 0, want2.size, nblocks=4), want2)
        st = s.stats()
        assert st["host_reads"] > 0 and st["host_map_reads"] == 0

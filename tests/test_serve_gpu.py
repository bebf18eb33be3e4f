"""The served form: a persistent device loop over a request ring gives each
request the oracle's answer (XXH64 of the range, dictionary tokens of the
range, bytes written), under a pool small enough to evict, with
memory-gated admission; written ranges land in the output files."""
import errno
import os

import numpy as np
import pytest

import gpufs_gb300 as g
from gpufs_gb300 import datagen
from oracle import oracle

pytestmark = pytest.mark.gpu


def _setup(d, seed):
    rng = np.random.default_rng(seed)
    voc = datagen.vocab(2000, seed=seed)
    sizes = [0, 100, 4096, 70000, 300001, 1 << 20, 2 * (1 << 20) + 13, 5 * (1 << 20) + 1]
    paths = []
    for i, n in enumerate(sizes):
        p = os.path.join(d, "s%02d.dat" % i)
        if i % 2:
            datagen.uniform_bytes(p, n, seed=seed + i)
        else:
            datagen.zipf_files([p], [n], voc, s=1.1, seed=seed + i)
        paths.append(p)
    dpath = os.path.join(d, "sdict.gpu")
    datagen.dictionary(dpath, voc, 700, seed=seed)
    outs = [os.path.join(d, "o%d.out" % i) for i in range(2)]
    return paths, dpath, outs, rng


def _dict_words(dpath):
    raw = open(dpath, "rb").read()
    recs = [raw[i:i + 32].split(b"\0", 1)[0] for i in range(0, len(raw), 32)]
    first = {}
    for i, w in enumerate(recs):
        if w and w not in first:
            first[w] = i
    return raw, sorted(first.values())


def _grep_tokens(raw_dict, first_idx, data):
    c = oracle.grep_counts(raw_dict, [data], mode="fast")
    return int(c[first_idx, 0].sum())


def _requests(paths, outs, rng, n, spread_ns):
    reqs = np.zeros(n, dtype=g.SERVE_REQ)
    sizes = [os.path.getsize(p) for p in paths]
    wpos = [0, 0]
    for k in range(n):
        op = [g.SV_READ, g.SV_READ, g.SV_GREP, g.SV_WRITE][k % 4]
        if op == g.SV_WRITE:
            o = k % 2
            reqs[k] = (op, o, wpos[o], int(rng.integers(1, 300000)), 0)
            wpos[o] += 1 << 20  # disjoint regions, 16-byte aligned
        else:
            f = int(rng.integers(0, len(paths)))
            off = int(rng.integers(0, max(1, sizes[f] // 4096 + 2))) * 4096
            reqs[k] = (op, f, off, int(rng.integers(0, 800000)), 0)
    reqs["arrival_ns"] = np.sort(rng.integers(0, spread_ns + 1, n)) if spread_ns else 0
    return reqs


def _check(res, reqs, paths, raw_dict, first_idx):
    files = [np.fromfile(p, dtype=np.uint8) for p in paths]
    for k in range(reqs.size):
        r, q = res[k], reqs[k]
        assert r["status"] == 0, (k, q, r)
        assert r["complete_ns"] >= r["submit_ns"] >= q["arrival_ns"]
        if q["op"] == g.SV_WRITE:
            assert r["result"] == q["length"]
            continue
        data = files[q["file"]][q["offset"]:q["offset"] + q["length"]]
        if q["op"] == g.SV_READ:
            assert r["result"] == oracle.xxh64(data), (k, q)
        else:
            assert r["result"] == _grep_tokens(raw_dict, first_idx, data.tobytes()), (k, q)


@pytest.mark.parametrize("spread_ms,pool_mb", [(0, 64), (20, 6)])
def test_served_requests_match_oracle(built, shm_dir, spread_ms, pool_mb):
    paths, dpath, outs, rng = _setup(shm_dir, seed=30 + spread_ms)
    raw_dict, first_idx = _dict_words(dpath)
    reqs = _requests(paths, outs, rng, 160, spread_ms * 1000000)
    with g.Session(log_page=16, pool_bytes=pool_mb << 20, max_files=64, timeout_s=30) as s:
        with g.Server(s, dpath, paths, outs) as sv:
            res = sv.run(reqs, inflight_pages=(pool_mb << 20) // (2 << 16))
            _check(res, reqs, paths, raw_dict, first_idx)
            res2 = sv.run(reqs[:40])  # a second run on the same server
            _check(res2, reqs[:40], paths, raw_dict, first_idx)
        assert s.last_error() == 0
    # the writes are in the output files once they are closed (write-back)
    for k in np.nonzero(reqs["op"] == g.SV_WRITE)[0]:
        q = reqs[k]
        got = np.fromfile(outs[q["file"]], dtype=np.uint8)[q["offset"]:q["offset"] + q["length"]]
        want = g.serve_pattern(int(q["offset"]), int(q["length"]), int(k))
        # the second run rewrote requests 0..39 with the same ids: same bytes
        assert np.array_equal(got, want), k


def test_served_any_offset(built, shm_dir):
    """Read and grep requests start at any byte (as gread does); pieces cross
    page boundaries at every alignment; writes must start 16-byte aligned."""
    paths, dpath, outs, rng = _setup(shm_dir, seed=50)
    raw_dict, first_idx = _dict_words(dpath)
    sizes = [os.path.getsize(p) for p in paths]
    reqs = np.zeros(64, dtype=g.SERVE_REQ)
    for k in range(63):
        f = 5 + k % 3
        op = g.SV_READ if k % 2 == 0 else g.SV_GREP
        off = int(rng.integers(0, sizes[f]))
        if k < 16:  # just before a 64 KiB page boundary, every alignment
            off = 65536 * (1 + k % 4) - 1 - k
        reqs[k] = (op, f, off, int(rng.integers(1, 300000)), 0)
    reqs[63] = (g.SV_WRITE, 0, 7, 100, 0)
    with g.Session(log_page=16, pool_bytes=32 << 20, max_files=64, timeout_s=30) as s:
        with g.Server(s, dpath, paths, outs) as sv:
            res = sv.run(reqs)
    assert res[63]["status"] == -errno.EINVAL
    _check(res[:63], reqs[:63], paths, raw_dict, first_idx)


@pytest.mark.parametrize("pool_mb", [64, 8])
def test_served_split_greps(built, shm_dir, pool_mb):
    """Greps longer than 1 MiB are split into parts that other warps take
    (a token is counted by the part its first letter falls in); many at once,
    at any offset, up to the end of the file, with and without eviction,
    mixed with reads: every count equals the oracle's."""
    paths, dpath, outs, rng = _setup(shm_dir, seed=70)
    raw_dict, first_idx = _dict_words(dpath)
    sizes = [os.path.getsize(p) for p in paths]
    reqs = np.zeros(48, dtype=g.SERVE_REQ)
    for k in range(48):
        f = [5, 6, 7][k % 3]
        off = int(rng.integers(0, sizes[f] // 3))
        length = int(rng.integers((1 << 20) + 1, 5 << 20))
        if k % 8 == 7:
            length = sizes[f]  # runs to the end of the file
        reqs[k] = (g.SV_GREP if k % 4 else g.SV_READ, f, off, length, 0)
    with g.Session(log_page=16, pool_bytes=pool_mb << 20, max_files=64, timeout_s=30) as s:
        with g.Server(s, dpath, paths, outs) as sv:
            res = sv.run(reqs, inflight_pages=(pool_mb << 20) // (2 << 16))
        assert s.last_error() == 0
    _check(res, reqs, paths, raw_dict, first_idx)


def test_serving_warps_are_resident(built, shm_dir):
    """A run uses whole blocks of 8 serving warps per SM, no more than the
    device holds at once (a persistent block that is not resident would
    serve nothing until others leave)."""
    paths, dpath, outs, _ = _setup(shm_dir, seed=90)
    with g.Session(log_page=16, pool_bytes=32 << 20, max_files=64, timeout_s=30) as s:
        with g.Server(s, dpath, paths, outs) as sv:
            got = [sv.warps_per_sm(w) for w in (1, 8, 16, 24, 32, 64)]
    assert all(w % 8 == 0 and 8 <= w <= max(8, asked) for w, asked in zip(got, (1, 8, 16, 24, 32, 64)))
    assert got == sorted(got) and got[1] == 8 and got[-1] < 64


def test_device_service_histogram(built, shm_dir):
    """The served kernel counts every request's device service time (from
    the take of its request to its completion) in a log2 histogram: one
    count per request, none below 256 ns or above 2**40 ns, and the device
    time of the slowest bucket no longer than the host-measured latency of
    the slowest request."""
    paths, dpath, outs, rng = _setup(shm_dir, seed=95)
    reqs = _requests(paths, outs, rng, 120, 0)
    with g.Session(log_page=16, pool_bytes=64 << 20, max_files=64, timeout_s=30) as s:
        with g.Server(s, dpath, paths, outs) as sv:
            res = sv.run(reqs)
            hist = sv.service_hist()
    assert hist.sum() == reqs.size
    nz = np.nonzero(hist)[0]
    assert nz.min() >= 8 and nz.max() <= 40
    host_max_ns = int((res["complete_ns"].astype(np.int64) - reqs["arrival_ns"].astype(np.int64)).max())
    assert 2 ** int(nz.max()) <= host_max_ns

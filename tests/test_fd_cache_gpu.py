"""More open files than the process may hold host fds for: the host closes
idle slots' fds past its open-file limit and reopens them by name when a
request needs one, so a plan or a server over thousands of files gives the
oracle's answers while the process stays under its limit -- with registered
file mappings (mapped reads need no fd) and without them (every miss is a
pread on a reopened fd), and for write-backs to evicted output files."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import gpufs_gb300 as g
from gpufs_gb300 import datagen
from oracle import oracle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, os, resource, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import gpufs_gb300 as g
d, file_map, limit = sys.argv[2], sys.argv[3] == "1", int(sys.argv[4])
paths = json.load(open(os.path.join(d, "paths.json")))
outs = [os.path.join(d, "o%d.out" % i) for i in range(3)]
soft, hard = resource.getrlimit(resource.RLIMIT_NOFILE)
resource.setrlimit(resource.RLIMIT_NOFILE, (limit, hard))
out = {}
with g.Session(log_page=16, pool_bytes=96 << 20, max_files=4096, timeout_s=30, file_map=file_map) as s:
    with g.Grep(s, os.path.join(d, "dict.gpu"), paths) as gr:
        out["fds_open"] = len(os.listdir("/proc/self/fd"))
        xxh, _ = gr.batch()
        out["xxh"] = [str(x) for x in xxh]
        out["counts_sum"] = [int(x) for x in gr.counts().sum(axis=0)]
    reqs = np.load(os.path.join(d, "reqs.npy"))
    with g.Server(s, os.path.join(d, "dict.gpu"), paths, outs) as sv:
        out["fds_serving"] = len(os.listdir("/proc/self/fd"))
        res = sv.run(reqs, inflight_pages=300)
        out["status"] = [int(x) for x in res["status"]]
        out["result"] = [str(int(x)) for x in res["result"]]
    st = s.stats()
    out["host_map_reads"] = int(st["host_map_reads"])
    out["last_error"] = int(s.last_error())
print("RESULT " + json.dumps(out))
"""


@pytest.mark.parametrize("file_map", [True, False])
def test_more_files_than_host_fds(built, shm_dir, file_map):
    rng = np.random.default_rng(77)
    voc = datagen.vocab(1500, seed=77)
    n = 1500
    sizes = [int(x) for x in rng.integers(0, 200000, n)]
    sizes[:4] = [0, 1, 65536, 131072 + 5]
    paths = []
    for i, sz in enumerate(sizes):
        p = os.path.join(shm_dir, "f%04d.dat" % i)
        if i % 2:
            datagen.uniform_bytes(p, sz, seed=1000 + i)
        else:
            datagen.zipf_files([p], [sz], voc, s=1.1, seed=1000 + i)
        paths.append(p)
    dpath = os.path.join(shm_dir, "dict.gpu")
    datagen.dictionary(dpath, voc, 500, seed=77)
    with open(os.path.join(shm_dir, "paths.json"), "w") as f:
        json.dump(paths, f)
    # requests: reads spread over every file, then writes to the outputs
    n_req = 600
    reqs = np.zeros(n_req, dtype=g.SERVE_REQ)
    for k in range(n_req):
        if k % 10 == 9:
            reqs[k] = (g.SV_WRITE, k % 3, (k // 3) * 65536, int(rng.integers(1, 65536)), 0)
        else:
            fi = int(rng.integers(0, n))
            off = int(rng.integers(0, sizes[fi] // 4096 + 1)) * 4096
            reqs[k] = (g.SV_READ, fi, off, int(rng.integers(1, 100000)), 0)
    np.save(os.path.join(shm_dir, "reqs.npy"), reqs)

    limit = 512  # the session keeps at most half of it for file slots
    cp = subprocess.run([sys.executable, "-c", CHILD, ROOT, shm_dir, "1" if file_map else "0", str(limit)],
                        capture_output=True, text=True, timeout=600)
    assert cp.returncode == 0, cp.stdout[-2000:] + cp.stderr[-4000:]
    line = [x for x in cp.stdout.splitlines() if x.startswith("RESULT ")][-1]
    out = json.loads(line[len("RESULT "):])
    assert out["last_error"] == 0
    assert out["fds_open"] < limit and out["fds_serving"] < limit, out

    files = [np.fromfile(p, dtype=np.uint8) for p in paths]
    assert [int(x) for x in out["xxh"]] == oracle.xxh64_many(files)
    want = oracle.grep_counts(open(dpath, "rb").read(), [f.tobytes() for f in files], mode="fast")
    assert out["counts_sum"] == [int(x) for x in want.sum(axis=0)]
    for k in range(n_req):
        q = reqs[k]
        assert out["status"][k] == 0, (k, q)
        if q["op"] == g.SV_WRITE:
            assert int(out["result"][k]) == int(q["length"])
        else:
            data = files[q["file"]][q["offset"]:q["offset"] + q["length"]]
            assert int(out["result"][k]) == oracle.xxh64(data), (k, q)
    for k in np.nonzero(reqs["op"] == g.SV_WRITE)[0]:
        q = reqs[k]
        got = np.fromfile(os.path.join(shm_dir, "o%d.out" % q["file"]), dtype=np.uint8)
        got = got[q["offset"]:q["offset"] + q["length"]]
        assert np.array_equal(got, g.serve_pattern(int(q["offset"]), int(q["length"]), int(k))), k
    if file_map:
        assert out["host_map_reads"] > 0
    else:
        assert out["host_map_reads"] == 0

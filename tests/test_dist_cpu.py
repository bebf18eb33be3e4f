"""The N>1 path of bench.py on CPU: two gloo ranks (127.0.0.1), each a
replica.  The path shards by file with no exchange, so the only
cross-rank steps are the barrier around the timed region and the
max-over-ranks of the measured time; both are checked here."""
import os
import socket
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent("""
    import os, sys, json
    sys.path.insert(0, %r)
    import bench
    rank, ws, local, td = bench.dist()
    assert ws == 2 and td is not None
    bench.barrier(td)
    t = bench.allmax(td, 1.0 + rank)          # each rank's own time
    print(json.dumps({"rank": rank, "ws": ws, "max": t}))
    td.destroy_process_group()
""")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_gloo_ranks_barrier_and_max():
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD % ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(out.strip().splitlines()[-1])
    import json
    res = sorted((json.loads(o) for o in outs), key=lambda r: r["rank"])
    assert [r["rank"] for r in res] == [0, 1]
    assert all(r["ws"] == 2 and r["max"] == 2.0 for r in res)


def test_reference_arm_other_ranks_exit_quietly(tmp_path):
    """Under N>1 only rank 0 runs the reference arm; other ranks do no work."""
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="1")
    r = subprocess.run([sys.executable, "-c", textwrap.dedent("""
        import sys; sys.path.insert(0, %r)
        import bench
        class A: pass
        a = A(); a.steps = 1; a.warmup = 0; a.gpus = 2
        bench.run_reference(a, 1, 2, None, %r)
        print("ok")
    """) % (ROOT, str(tmp_path))], env=env, capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "ok"

"""Host logic of the Python binding (CPU only, with a fake native library
that records its calls): a Session closes its open Grep plans and Servers
before it ends, and a plan or server closed after its session has ended
makes no native call (the native objects went with the session)."""
import ctypes
import weakref

import gpufs_gb300 as g


class FakeLib:
    def __init__(self):
        self.calls = []

    def _open(self, name, ref, value):
        self.calls.append(name)
        ref._obj.value = value
        return 0

    def gfs_grep_open(self, sh, dpath, paths, n, ref):
        return self._open("gfs_grep_open", ref, 0x1000 + len(self.calls))

    def gfs_grep_info(self, h, info, n):
        self.calls.append("gfs_grep_info")
        return 0

    def gfs_grep_close(self, h):
        self.calls.append("gfs_grep_close")
        return 0

    def gfs_serve_open(self, sh, dpath, paths, n, outs, n_out, ref):
        return self._open("gfs_serve_open", ref, 0x2000 + len(self.calls))

    def gfs_serve_close(self, h):
        self.calls.append("gfs_serve_close")
        return 0

    def gfs_destroy(self, h):
        self.calls.append("gfs_destroy")
        return 0


def _session():
    s = object.__new__(g.Session)
    s._h = ctypes.c_void_p(0x55)
    s.L = FakeLib()
    s._children = weakref.WeakSet()
    return s


def test_session_close_closes_open_plans_and_servers_first():
    s = _session()
    gr = g.Grep(s, "/x/dict.gpu", ["/x/a.txt"])
    sv = g.Server(s, "/x/dict.gpu", ["/x/a.txt"], ["/x/out.bin"])
    s.close()
    calls = s.L.calls
    assert calls.count("gfs_grep_close") == 1 and calls.count("gfs_serve_close") == 1
    assert calls[-1] == "gfs_destroy" and calls.count("gfs_destroy") == 1
    # closing them again after the session ended makes no native call
    n = len(calls)
    gr.close()
    sv.close()
    s.close()
    assert len(s.L.calls) == n


def test_closed_plan_is_not_closed_twice():
    s = _session()
    with g.Grep(s, "/x/dict.gpu", ["/x/a.txt"]):
        pass
    s.close()
    assert s.L.calls.count("gfs_grep_close") == 1
    assert s.L.calls[-1] == "gfs_destroy"

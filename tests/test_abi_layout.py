"""The C ABI's layouts and constants, as a C compiler sees them, against the
Python binding: a small program built with gcc against include/ prints the
sizes, field offsets and #defines, and the ctypes structure, the numpy
record types and the Python constants must agree with them byte for byte.
Also pins the shared layouts' sizes that the device code and the host
runtime rely on (gfs_open_reply 32 B, gfs_req 136 B, gfs_frame 32 B) and
the 8-byte alignment of the 64-bit fields device code moves as one word."""
import ctypes
import os
import shutil
import subprocess

import pytest

import gpufs_gb300 as g
from gpufs_gb300 import costmodel

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_PROG = r"""
#include <stddef.h>
#include <stdio.h>
#include "fs_constants.h"
#include "gfs_types.h"
#include "gpufs_gb300.h"
#define P(name, v) printf("%s %lld\n", name, (long long)(v))
#define OFF(t, f) P(#t "." #f, offsetof(t, f))
int main(void) {
    P("sizeof.gfs_config", sizeof(gfs_config));
    OFF(gfs_config, log_page); OFF(gfs_config, max_files); OFF(gfs_config, pool_bytes);
    OFF(gfs_config, ring_slots); OFF(gfs_config, host_workers); OFF(gfs_config, staging_depth);
    OFF(gfs_config, flags); OFF(gfs_config, timeout_ns); OFF(gfs_config, device); OFF(gfs_config, pad1);
    P("sizeof.gfs_serve_req", sizeof(gfs_serve_req));
    OFF(gfs_serve_req, op); OFF(gfs_serve_req, file); OFF(gfs_serve_req, offset);
    OFF(gfs_serve_req, length); OFF(gfs_serve_req, arrival_ns);
    P("sizeof.gfs_serve_res", sizeof(gfs_serve_res));
    OFF(gfs_serve_res, result); OFF(gfs_serve_res, status); OFF(gfs_serve_res, pad);
    OFF(gfs_serve_res, submit_ns); OFF(gfs_serve_res, complete_ns);
    P("sizeof.gfs_open_reply", sizeof(gfs_open_reply));
    P("sizeof.gfs_req", sizeof(gfs_req));
    P("sizeof.gfs_frame", sizeof(gfs_frame));
    OFF(gfs_file, size); OFF(gfs_file, ctime_ns); OFF(gfs_file, map_dev);
    OFF(gfs_open_reply, size); OFF(gfs_open_reply, ctime_ns); OFF(gfs_open_reply, map_dev);
    OFF(gfs_req, offset); OFF(gfs_req, length); OFF(gfs_req, dev_addr); OFF(gfs_req, done_addr);
    P("GFS_CFG_NO_FILE_MAP", GFS_CFG_NO_FILE_MAP); P("GFS_CFG_RETAIN_CACHE", GFS_CFG_RETAIN_CACHE); P("GFS_CFG_HOST_TABLE", GFS_CFG_HOST_TABLE);
    P("GFS_NSTATS", GFS_NSTATS);
    P("GFS_XXH64_NOALLOC_MAX_FILES", GFS_XXH64_NOALLOC_MAX_FILES);
    P("GFS_SV_READ", GFS_SV_READ); P("GFS_SV_GREP", GFS_SV_GREP); P("GFS_SV_WRITE", GFS_SV_WRITE);
    P("GFS_CM_HIDDEN", GFS_CM_HIDDEN); P("GFS_CM_MAX_INPUTS", GFS_CM_MAX_INPUTS);
    P("GFS_ERRB_TIMEOUT", GFS_ERRB_TIMEOUT); P("GFS_ERRB_IO", GFS_ERRB_IO);
    P("GFS_ERRB_NOMEM", GFS_ERRB_NOMEM); P("GFS_ERRB_TABLE", GFS_ERRB_TABLE); P("GFS_ERRB_ARG", GFS_ERRB_ARG);
    P("O_GRDONLY", O_GRDONLY); P("O_GWRONLY", O_GWRONLY); P("O_GCREAT", O_GCREAT);
    P("O_GRDWR", O_GRDWR); P("O_GWRONCE", O_GWRONCE);
    return 0;
}
"""


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "layout.c", d / "layout"
    src.write_text(_PROG)
    subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (line.split() for line in out.splitlines())}


def test_config_struct_matches(c_layout):
    assert ctypes.sizeof(g.Config) == c_layout["sizeof.gfs_config"]
    for name, _ in g.Config._fields_:
        assert getattr(g.Config, name).offset == c_layout["gfs_config." + name], name


@pytest.mark.parametrize("dtype,cname", [(g.SERVE_REQ, "gfs_serve_req"), (g.SERVE_RES, "gfs_serve_res")])
def test_serve_records_match(c_layout, dtype, cname):
    assert dtype.itemsize == c_layout["sizeof." + cname]
    for name in dtype.names:
        assert dtype.fields[name][1] == c_layout[cname + "." + name], name


def test_constants_match(c_layout):
    assert g.CFG_NO_FILE_MAP == c_layout["GFS_CFG_NO_FILE_MAP"]
    assert g.CFG_RETAIN_CACHE == c_layout["GFS_CFG_RETAIN_CACHE"]
    assert g.CFG_HOST_TABLE == c_layout["GFS_CFG_HOST_TABLE"]
    assert len(g.STAT_NAMES) == c_layout["GFS_NSTATS"]
    assert g.XXH64_NOALLOC_MAX_FILES == c_layout["GFS_XXH64_NOALLOC_MAX_FILES"]
    assert (g.SV_READ, g.SV_GREP, g.SV_WRITE) == (c_layout["GFS_SV_READ"], c_layout["GFS_SV_GREP"],
                                                  c_layout["GFS_SV_WRITE"])
    assert (costmodel.HIDDEN, costmodel.MAX_INPUTS) == (c_layout["GFS_CM_HIDDEN"], c_layout["GFS_CM_MAX_INPUTS"])
    assert (g.ERR_TIMEOUT, g.ERR_IO, g.ERR_NOMEM, g.ERR_TABLE, g.ERR_ARG) == tuple(
        c_layout["GFS_ERRB_" + n] for n in ("TIMEOUT", "IO", "NOMEM", "TABLE", "ARG"))
    for n in ("O_GRDONLY", "O_GWRONLY", "O_GCREAT", "O_GRDWR", "O_GWRONCE"):
        assert getattr(g, n) == c_layout[n], n


def test_shared_layout_sizes(c_layout):
    assert c_layout["sizeof.gfs_open_reply"] == 32
    assert c_layout["sizeof.gfs_req"] == 136
    assert c_layout["sizeof.gfs_frame"] == 32
    # 64-bit fields that device code loads and stores as single 64-bit words
    for k in ("gfs_file.size", "gfs_file.ctime_ns", "gfs_file.map_dev", "gfs_open_reply.size",
              "gfs_open_reply.ctime_ns", "gfs_open_reply.map_dev", "gfs_req.offset", "gfs_req.length",
              "gfs_req.dev_addr", "gfs_req.done_addr"):
        assert c_layout[k] % 8 == 0, k

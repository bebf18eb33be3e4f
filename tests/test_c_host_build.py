"""A plain C host program over the C ABI (the way a cgo / JNI / ctypes
binding would call it) compiles as C11
against include/gpufs_gb300.h with warnings as errors and links against
libgpufs_gb300.so.  CPU only: nothing is run."""
import os
import shutil
import subprocess

import pytest

from gpufs_gb300 import build as gbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_PROG = r"""
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include "gpufs_gb300.h"

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    gfs_config c;
    gfs_default_config(&c);
    c.log_page = 20;
    c.pool_bytes = 4ull << 30;
    c.flags |= GFS_CFG_RETAIN_CACHE;
    gfs_ctx* fs;
    if (gfs_create(&c, &fs)) return 1;
    printf("retained pages %lld\n", gfs_retained_pages(fs));
    const char* files[] = {argv[2]};
    const int n_words = 20000;
    uint32_t* counts = (uint32_t*)malloc((size_t)n_words * sizeof(uint32_t));
    int rc = gfs_grep_text(fs, argv[1], files, 1, counts, 0);
    unsigned long long st[GFS_NSTATS];
    gfs_get_stats(fs, st, GFS_NSTATS);
    unsigned char buf[4096];
    long long got = gfs_pread(fs, argv[2], 0, sizeof buf, buf, 1, 256);
    gfs_destroy(fs);
    gfs_release_retained();
    free(counts);
    return rc < 0 || got < 0;
}
"""


def test_c_program_compiles_and_links(built, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src, exe = tmp_path / "host.c", tmp_path / "host"
    src.write_text(_PROG)
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(gbuild.nvcc())), "lib64")
    r = subprocess.run([cc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"), str(src),
                        "-o", str(exe), "-L" + gbuild.OUT, "-lgpufs_gb300", "-L" + cuda_lib, "-lcudart",
                        "-Wl,-rpath," + gbuild.OUT], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-3000:]

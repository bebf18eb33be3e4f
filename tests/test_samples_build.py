"""The reference's in-scope samples rebuild unchanged against this library.

memcopy (samples/memcopy/cp.cu), grep_text (samples/grep_text/fs.cu, which
includes grep_text_gpu.cu) and bigmatrix_mmap (samples/bigmatrix_mmap/fs.cu,
which includes bigmatrix_mmap.cu) are compiled from the reference tree, as
they stand, with relocatable device code against include/ and linked with
libgpufs.a -- the build recipe of the reference's sample Makefiles
(samples/grep_text/Makefile:27-39) with this library in place of
libgpufs.  CPU only: the binaries are not run here.  Skipped where the
reference tree is absent.
"""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

import pytest

from gpufs_gb300 import build as gbuild

from oracle import oracle

REF = oracle.reference_root()
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SAMPLES = ["memcopy/cp.cu", "grep_text/fs.cu", "bigmatrix_mmap/fs.cu"]

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "samples")),
                                reason="reference samples not present")


def _build(sample, outdir):
    d = os.path.dirname(sample)
    src = os.path.join(REF, "samples", sample)
    obj = os.path.join(outdir, d + ".o")
    exe = os.path.join(outdir, d + ".bin")
    nv = gbuild.nvcc()
    arch = gbuild.ARCH
    c = subprocess.run([nv] + arch + ["-rdc=true", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                                      "-I" + os.path.dirname(src), "-c", src, "-o", obj],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if c.returncode:
        return sample, "compile", c.stdout
    lk = subprocess.run([nv] + arch + ["-rdc=true", obj, os.path.join(gbuild.OUT, "libgpufs.a"), "-o", exe,
                                       "-lcudart"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if lk.returncode:
        return sample, "link", lk.stdout
    return sample, "ok", ""


def test_samples_compile_and_link_unchanged(built, tmp_path):
    with ThreadPoolExecutor(len(SAMPLES)) as ex:
        res = list(ex.map(lambda s: _build(s, str(tmp_path)), SAMPLES))
    bad = [(s, what, log[-2000:]) for s, what, log in res if what != "ok"]
    assert not bad, bad

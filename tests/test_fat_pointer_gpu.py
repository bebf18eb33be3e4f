"""Fat pointers (gvmmap/FatPointer/TLB, the interface of the reference's
fat_pointer.cu.h) in a program built the way GPUfs programs are: compiled
with relocatable device code against include/ and linked with libgpufs.a.
The kernel reads a file through fat pointers (grid stride across 64 KiB
pages, scattered moveTo, backwards steps, operator[]) and writes a
transformed copy through a write-once fat pointer; the program checks the
values and the output file (tests/gpu_src/fat_pointer_test.cu)."""
import os
import subprocess

import numpy as np
import pytest

from gpufs_gb300 import build as gbuild

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _pattern(n):
    i = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = i * np.uint64(0x9E3779B97F4A7C15) + np.uint64(0x1234567)
        z ^= z >> np.uint64(29)
        return ((z * np.uint64(0xBF58476D1CE4E5B9)) >> np.uint64(32)).astype(np.uint32)


@pytest.fixture(scope="module")
def fp_exe(built, tmp_path_factory):
    d = tmp_path_factory.mktemp("fp")
    src = os.path.join(HERE, "gpu_src", "fat_pointer_test.cu")
    obj, exe = str(d / "fp.o"), str(d / "fp.bin")
    nv = gbuild.nvcc()
    subprocess.run([nv] + gbuild.ARCH + ["-rdc=true", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-c", src,
                                         "-o", obj], check=True)
    subprocess.run([nv] + gbuild.ARCH + ["-rdc=true", obj, os.path.join(gbuild.OUT, "libgpufs.a"), "-o", exe,
                                         "-lcudart"], check=True)
    return exe


@pytest.mark.parametrize("n", [3 * 16384 + 777, 16384, 5])
def test_fat_pointers_read_and_write_through_the_cache(fp_exe, shm_dir, n):
    src = os.path.join(shm_dir, "fp_in.bin")
    out = os.path.join(shm_dir, "fp_out.bin")
    data = _pattern(n)
    data.tofile(src)
    cp = subprocess.run([fp_exe, src, out], capture_output=True, text=True, timeout=300)
    assert cp.returncode == 0, cp.stdout + cp.stderr
    assert "OK" in cp.stdout
    got = np.fromfile(out, dtype=np.uint32)
    with np.errstate(over="ignore"):
        assert np.array_equal(got, data * np.uint32(3) + np.uint32(1))

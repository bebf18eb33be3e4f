"""Programs written against the reference's device and host API the way its
samples use it, built like GPUfs programs (relocatable device code against
include/, linked with libgpufs.a) and run on the GPU
(tests/gpu_src/api_programs_test.cu): a page-by-page gread/gwrite copy into
a new write-once file through a shared-memory buffer (the pattern of
samples/memcopy/cp.cu:73-108), and gmsync of a mapped page of an O_GRDWR
file, checked on the host while the kernel still holds the file open
(libgpufs/fs_calls.cu:804-843)."""
import os
import subprocess

import numpy as np
import pytest

from gpufs_gb300 import build as gbuild
from gpufs_gb300 import datagen
from oracle import oracle

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PAGE = 16384  # the program's FS_LOGBLOCKSIZE 14


@pytest.fixture(scope="module")
def api_exe(built, tmp_path_factory):
    d = tmp_path_factory.mktemp("api")
    src = os.path.join(HERE, "gpu_src", "api_programs_test.cu")
    obj, exe = str(d / "api.o"), str(d / "api.bin")
    nv = gbuild.nvcc()
    subprocess.run([nv] + gbuild.ARCH + ["-rdc=true", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-c", src,
                                         "-o", obj], check=True)
    subprocess.run([nv] + gbuild.ARCH + ["-rdc=true", obj, os.path.join(gbuild.OUT, "libgpufs.a"), "-o", exe,
                                         "-lcudart"], check=True)
    return exe


@pytest.mark.parametrize("n", [21 * PAGE + 1234, PAGE, 3, 0])
def test_copy_program(api_exe, shm_dir, n):
    src = os.path.join(shm_dir, "c_in.bin")
    dst = os.path.join(shm_dir, "c_out.bin")
    datagen.uniform_bytes(src, n, seed=n + 1)
    cp = subprocess.run([api_exe, "copy", src, dst], capture_output=True, text=True, timeout=300)
    assert cp.returncode == 0, cp.stdout + cp.stderr
    assert "OK" in cp.stdout
    a = np.fromfile(src, dtype=np.uint8)
    b = np.fromfile(dst, dtype=np.uint8)
    assert b.size == a.size and oracle.xxh64(b) == oracle.xxh64(a)


@pytest.mark.parametrize("size,n", [(200000, 4000), (PAGE, PAGE), (1000, 1000)])
def test_gmsync_writes_back_while_open(api_exe, shm_dir, size, n):
    """The host sees the first pattern after gmsync while the file is still
    open on the device (the program checks it); the second pattern reaches
    the file at close; bytes past the written ones keep their values.  The
    program maps a whole page with write flags, and a write mapping makes its
    range part of the file (the reference raises the page's content size to
    the mapped range, libgpufs/fs_calls.cu:459-460, and gmsync writes that
    many bytes back), so a shorter file grows to the page, zero filled."""
    p = os.path.join(shm_dir, "ms.bin")
    datagen.uniform_bytes(p, size, seed=77)
    before = np.fromfile(p, dtype=np.uint8)
    cp = subprocess.run([api_exe, "msync", p, str(n)], capture_output=True, text=True, timeout=300)
    assert cp.returncode == 0, cp.stdout + cp.stderr
    after = np.fromfile(p, dtype=np.uint8)
    assert after.size == max(size, PAGE)
    assert np.array_equal(after[n:size], before[n:size])
    assert not after[size:].any()

"""The fat-pointer test program (gvmmap/FatPointer templates over include/)
compiles with relocatable device code and links against libgpufs.a, the way
GPUfs programs are built.  CPU only: it is run by the GPU tests."""
import os
import subprocess

from gpufs_gb300 import build as gbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fat_pointer_program_compiles_and_links(built, tmp_path):
    src = os.path.join(ROOT, "tests", "gpu_src", "fat_pointer_test.cu")
    obj, exe = str(tmp_path / "fp.o"), str(tmp_path / "fp.bin")
    nv = gbuild.nvcc()
    c = subprocess.run([nv] + gbuild.ARCH + ["-rdc=true", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-c",
                                             src, "-o", obj], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert c.returncode == 0, c.stdout[-3000:]
    lk = subprocess.run([nv] + gbuild.ARCH + ["-rdc=true", obj, os.path.join(gbuild.OUT, "libgpufs.a"), "-o", exe,
                                              "-lcudart"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert lk.returncode == 0, lk.stdout[-3000:]

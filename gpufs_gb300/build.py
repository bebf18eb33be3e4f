"""Build step for the native parts of gpufs_gb300 (in-tree, no cmake).

Compiles, in parallel:
  * the CUDA library (sm_103a, relocatable device code) into
    gpufs_gb300/_build/libgpufs_gb300.so (C ABI, include/gpufs_gb300.h) and
    gpufs_gb300/_build/libgpufs.a (for programs written against the
    reference's device API, linked with nvcc -rdc=true);
  * the seeded workload generator into gpufs_gb300/_build/libgfs_datagen.so.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
OUT = os.path.join(HERE, "_build")

CUDA_SOURCES = ["gfs_calls.cu", "gfs_runtime.cu", "gfs_workloads.cu", "gfs_grep.cu", "gfs_apps.cu",
                "gfs_bigmatrix.cu", "gfs_costmodel.cu"]
# Device-API translation units are linked as relocatable code into kernels of
# any block size (up to 1024 threads): cap them at 64 registers per thread.
# gfs_bigmatrix.cu is not capped: its kernel is bounded at 512 threads a
# block (__launch_bounds__) and uses the registers that leaves.
PER_FILE_FLAGS = {"gfs_calls.cu": ["-maxrregcount=64"], "gfs_workloads.cu": ["-maxrregcount=64"],
                  "gfs_runtime.cu": ["-maxrregcount=64"], "gfs_apps.cu": ["-maxrregcount=64"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-rdc=true", "-std=c++17", "-Xcompiler", "-fPIC",
              "-I" + INC, "-I" + CSRC, "--expt-relaxed-constexpr"]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def _headers():
    hs = []
    for d in (CSRC, INC):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                hs.append(os.path.join(d, f))
    return hs


def build(verbose=False, ptxas_v=False):
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    hdrs = _headers()
    srcs = [s for s in CUDA_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    jobs = []
    objs = []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, s.replace(".cu", ".o"))
        objs.append(obj)
        if not _newer(obj, [src] + hdrs):
            extra = ["-Xptxas", "-v"] if ptxas_v else []
            jobs.append([nv] + ARCH + NVCC_FLAGS + PER_FILE_FLAGS.get(s, []) + extra + ["-c", src, "-o", obj])
    dg_src = os.path.join(CSRC, "datagen.c")
    dg_so = os.path.join(OUT, "libgfs_datagen.so")
    if not _newer(dg_so, [dg_src]):
        jobs.append(["gcc", "-O2", "-shared", "-fPIC", "-pthread", "-ffp-contract=off", "-fno-math-errno",
                     "-o", dg_so, dg_src])
    logs = []
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    so = os.path.join(OUT, "libgpufs_gb300.so")
    if not _newer(so, objs):
        logs.append(_run([nv] + ARCH + ["-shared", "-rdc=true", "-Xcompiler", "-fPIC", "-o", so] + objs +
                         ["-lcudart"]))
    ar = os.path.join(OUT, "libgpufs.a")
    if not _newer(ar, objs):
        if os.path.exists(ar):
            os.remove(ar)
        logs.append(_run(["ar", "rcs", ar] + objs))
    if verbose:
        sys.stdout.write("".join(logs))
    return so


if __name__ == "__main__":
    build(verbose=True, ptxas_v="-v" in sys.argv)

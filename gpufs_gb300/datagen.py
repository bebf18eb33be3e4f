"""Seeded synthetic inputs for the file-system workloads (see csrc/datagen.c).

The reference's inputs (a Shakespeare corpus, its word list, random
matrices) are replaced by files with the shapes and value distributions of
the benchmark configurations:
  memcopy   one file of uniform random bytes;
  grep_text N text files of Zipf(s) words over a random lowercase vocabulary
            (lengths 3-12), single spaces, a newline every ~80 characters, plus
            a dictionary of 32-byte NUL-padded records (dict.gpu format);
  bigmatrix an N(0,1) FP32 row-major matrix and vector;
  batched   files with log-uniform sizes, half random bytes, half Zipf text.
"""
import ctypes
import os

import numpy as np

from . import BUILD_DIR

_dg = None


def dg():
    global _dg
    if _dg is None:
        p = os.path.join(BUILD_DIR, "libgfs_datagen.so")
        if not os.path.exists(p):
            raise RuntimeError("datagen library missing: %s" % p)
        L = ctypes.CDLL(p)
        u64 = ctypes.c_uint64
        L.dg_uniform_bytes.argtypes = [ctypes.c_char_p, u64, u64, ctypes.c_int]
        L.dg_vocab.argtypes = [u64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.dg_zipf_files.argtypes = [ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(u64), ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_int, ctypes.c_double, u64, ctypes.c_int]
        L.dg_dictionary.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, u64]
        L.dg_normal_f32.argtypes = [ctypes.c_char_p, u64, u64, ctypes.c_int]
        L.dg_loguniform_sizes.argtypes = [u64, ctypes.c_int, u64, u64, ctypes.POINTER(u64)]
        L.dg_coin.argtypes = [u64, u64]
        _dg = L
    return _dg


def _threads():
    return max(1, min(32, os.cpu_count() or 1))


def uniform_bytes(path, nbytes, seed=0x6770756673):
    if dg().dg_uniform_bytes(os.fsencode(path), nbytes, seed, _threads()) != 0:
        raise OSError("dg_uniform_bytes failed for %s" % path)


def vocab(n=50000, seed=0x766f6361, minlen=3, maxlen=12):
    buf = np.zeros(n * 16, dtype=np.uint8)
    if dg().dg_vocab(seed, n, minlen, maxlen, buf.ctypes.data) != 0:
        raise RuntimeError("dg_vocab failed")
    return buf


def zipf_files(paths, sizes, voc, s=1.1, seed=0x7a697066):
    n = len(paths)
    arr_p = (ctypes.c_char_p * n)(*[os.fsencode(p) for p in paths])
    arr_s = (ctypes.c_uint64 * n)(*sizes)
    nv = voc.size // 16
    if dg().dg_zipf_files(arr_p, arr_s, n, voc.ctypes.data, nv, s, seed, _threads()) != 0:
        raise OSError("dg_zipf_files failed")


def dictionary(path, voc, n_words, seed=0x64696374):
    if dg().dg_dictionary(os.fsencode(path), voc.ctypes.data, voc.size // 16, n_words, seed) != 0:
        raise OSError("dg_dictionary failed")


def normal_f32(path, count, seed=0x4e4f524d):
    if dg().dg_normal_f32(os.fsencode(path), count, seed, _threads()) != 0:
        raise OSError("dg_normal_f32 failed")


def loguniform_sizes(n, lo, hi, seed=0x73697a65):
    out = (ctypes.c_uint64 * n)()
    dg().dg_loguniform_sizes(seed, n, lo, hi, out)
    return [int(v) for v in out]


def coin(seed, i):
    return int(dg().dg_coin(seed, i))


def grep_corpus(dirpath, n_files, total_bytes, n_vocab=50000, n_dict=20000, seed=1, s=1.1):
    """Write the grep_text inputs under dirpath; returns (file paths, dict path)."""
    os.makedirs(dirpath, exist_ok=True)
    voc = vocab(n_vocab, seed=0x766f6361 ^ seed)
    per = total_bytes // n_files
    sizes = [per] * n_files
    sizes[-1] += total_bytes - per * n_files
    paths = [os.path.join(dirpath, "c%03d.txt" % i) for i in range(n_files)]
    zipf_files(paths, sizes, voc, s=s, seed=0x7a697066 ^ seed)
    dpath = os.path.join(dirpath, "dict.gpu")
    dictionary(dpath, voc, n_dict, seed=0x64696374 ^ seed)
    return paths, dpath

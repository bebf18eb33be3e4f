"""The seeded workload generator: determinism and distributions (CPU)."""
import json
import os

import numpy as np

from gpufs_gb300 import datagen
from oracle import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "datagen_golden.json")


def test_generator_matches_golden(built, tmp_path):
    import importlib.util
    spec = importlib.util.spec_from_file_location("mk", os.path.join(os.path.dirname(GOLDEN), "make_golden.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    got = mk.datagen_case(str(tmp_path))
    want = json.load(open(GOLDEN))
    assert got == want


def test_vocab_and_corpus_shape(built, tmp_path):
    voc = datagen.vocab(2000, seed=5)
    words = [bytes(voc[i * 16:(i + 1) * 16]).rstrip(b"\0") for i in range(2000)]
    assert len(set(words)) == 2000
    assert all(3 <= len(w) <= 12 and w.isalpha() and w.islower() for w in words)
    p = str(tmp_path / "c.txt")
    datagen.zipf_files([p], [200000], voc, s=1.1, seed=9)
    data = open(p, "rb").read()
    assert len(data) == 200000
    assert set(data) <= set(b"abcdefghijklmnopqrstuvwxyz \n")
    lines = data.split(b"\n")
    assert max(len(l) for l in lines[:-1]) <= 80
    toks = data.split()
    # Zipf(1.1): the most frequent word is far above uniform frequency
    _, cnt = np.unique(np.array(toks, dtype=object), return_counts=True)
    assert cnt.max() / len(toks) > 0.05


def test_dictionary_records(built, tmp_path):
    voc = datagen.vocab(1000, seed=5)
    p = str(tmp_path / "d.gpu")
    datagen.dictionary(p, voc, 300, seed=3)
    b = open(p, "rb").read()
    assert len(b) == 300 * 32
    recs = [b[i * 32:(i + 1) * 32] for i in range(300)]
    names = [r.rstrip(b"\0") for r in recs]
    assert len(set(names)) == 300
    assert all(r[len(n):] == b"\0" * (32 - len(n)) for r, n in zip(recs, names))


def test_normal_moments(built, tmp_path):
    p = str(tmp_path / "n.f32")
    datagen.normal_f32(p, 1 << 20, seed=1)
    a = np.fromfile(p, dtype=np.float32)
    assert abs(float(a.mean())) < 0.01 and abs(float(a.std()) - 1.0) < 0.01


def test_loguniform_sizes(built):
    s = datagen.loguniform_sizes(4096, 4096, 64 << 20, seed=2)
    assert min(s) >= 4096 and max(s) <= 64 << 20
    total = sum(s)
    # E[size] for log-uniform on [4 KiB, 64 MiB] ~ 6.9 MiB -> ~28 GB for 4096 files
    assert 10e9 < total < 50e9

"""Regenerates the committed golden values in this directory.

  reference_fixture_counts.json  grep counts of the reference's own inputs
      (samples/grep_text/input/dict.gpu, first 4000 records, over
      samples/grep_text/input/pg100.txt.small), computed by the faithful
      oracle whose matcher is pinned to the reference's match_string; only the
      total and an XXH64 digest of the count matrix are stored.
  ref_dict_4000.gpu, ref_pg100_small.txt  those two inputs, copied byte for
      byte from the reference tree (the dictionary cut to its first 4000
      records), so the GPU tests can run the scan on them where the
      reference tree is absent.
  datagen_golden.json  XXH64 digests of small seeded inputs from the
      workload generator, and the faithful grep counts over them.

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import __graft_entry__  # noqa: E402
from gpufs_gb300 import datagen  # noqa: E402
from oracle import oracle  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def datagen_case(d):
    out = {}
    p = os.path.join(d, "u.bin")
    datagen.uniform_bytes(p, 100003, seed=7)
    out["uniform_100003_seed7"] = "%016x" % oracle.xxh64(open(p, "rb").read())
    voc = datagen.vocab(500, seed=11)
    out["vocab_500_seed11"] = "%016x" % oracle.xxh64(voc.tobytes())
    paths = [os.path.join(d, "c%d.txt" % i) for i in range(3)]
    datagen.zipf_files(paths, [50000, 60001, 7], voc, s=1.1, seed=13)
    out["zipf_files"] = ["%016x" % oracle.xxh64(open(q, "rb").read()) for q in paths]
    dp = os.path.join(d, "dict.gpu")
    datagen.dictionary(dp, voc, 120, seed=17)
    recs = open(dp, "rb").read()
    out["dict_120_seed17"] = "%016x" % oracle.xxh64(recs)
    counts = oracle.grep_counts(recs, [open(q, "rb").read() for q in paths], mode="faithful")
    out["grep_counts_faithful"] = "%016x" % oracle.xxh64(counts.astype("<u4").tobytes())
    out["grep_counts_total"] = int(counts.sum())
    np_ = os.path.join(d, "n.f32")
    datagen.normal_f32(np_, 10001, seed=19)
    out["normal_10001_seed19"] = "%016x" % oracle.xxh64(open(np_, "rb").read())
    out["loguniform_sizes"] = datagen.loguniform_sizes(16, 4096, 64 << 20, seed=23)
    return out


def main():
    __graft_entry__.build()
    with tempfile.TemporaryDirectory() as d:
        g = datagen_case(d)
    with open(os.path.join(HERE, "datagen_golden.json"), "w") as f:
        json.dump(g, f, indent=1)
    root = oracle.reference_root()
    dpath = os.path.join(root, "samples/grep_text/input/dict.gpu")
    tpath = os.path.join(root, "samples/grep_text/input/pg100.txt.small")
    if os.path.exists(dpath):
        recs = open(dpath, "rb").read()[:32 * 4000]
        text = open(tpath, "rb").read()
        with open(os.path.join(HERE, "ref_dict_4000.gpu"), "wb") as f:
            f.write(recs)
        with open(os.path.join(HERE, "ref_pg100_small.txt"), "wb") as f:
            f.write(text)
        c = oracle.grep_counts(recs, [text], mode="faithful")
        with open(os.path.join(HERE, "reference_fixture_counts.json"), "w") as f:
            json.dump({"records": 4000, "total": int(c.sum()),
                       "xxh64": "%016x" % oracle.xxh64(c.astype("<u4").tobytes())}, f, indent=1)


if __name__ == "__main__":
    main()

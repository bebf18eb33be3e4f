"""The oracle pinned against the reference and known answers (CPU only)."""
import ctypes
import ctypes.util
import json
import os

import numpy as np
import pytest

from oracle import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _libxxhash():
    for name in ("libxxhash.so.0", ctypes.util.find_library("xxhash")):
        if not name:
            continue
        try:
            lib = ctypes.CDLL(name)
            lib.XXH64.restype = ctypes.c_uint64
            lib.XXH64.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint64]
            return lib
        except OSError:
            continue
    return None


def test_xxh64_known_answers(built):
    # values obtained by calling the system libxxhash 0.8.2 (XXH64 export)
    assert oracle.xxh64(b"") == 0xEF46DB3751D8E999
    assert oracle.xxh64(b"abc") == 0x44BC2CF5AD770999


def test_xxh64_vs_system_libxxhash(built):
    lib = _libxxhash()
    if lib is None:
        pytest.skip("system libxxhash not present")
    rng = np.random.default_rng(1)
    for n in list(range(0, 130)) + [1000, 4096, 65536 + 7, 1 << 20]:
        a = rng.integers(0, 256, n, dtype=np.uint8)
        for seed in (0, 1, 0x9E3779B97F4A7C15):
            want = lib.XXH64(a.ctypes.data if n else None, n, seed)
            assert oracle.xxh64(a, seed) == want, (n, seed)


def _word33(w):
    b = w.encode() if isinstance(w, str) else w
    assert len(b) <= 32
    return b + b"\0" * (33 - len(b))


def test_match_string_hand_example(built):
    data = b"the cat sat on the cat_ mat with a catalog; scat cat's cat\n\0"
    # tokens equal to "cat": 'cat', 'cat' (of cat's), 'cat'; not cat_, catalog, scat
    assert oracle.match_string(_word33("cat"), data) == 3
    assert oracle.match_string(_word33("cat_"), data) == 1
    assert oracle.match_string(_word33("s"), data) == 1
    assert oracle.match_string(_word33(""), data) == -1
    assert oracle.match_string(_word33("the"), b"the") == 0  # no delimiter after it
    assert oracle.match_string(_word33("the"), b"the\0") == 1


def _rand_text(rng, n, alphabet):
    return bytes(rng.choice(alphabet, n))


def test_match_string_vs_reference_code(built):
    ref = oracle.ref()
    if ref is None:
        pytest.skip("reference matcher not built (no reference tree on this machine)")
    rng = np.random.default_rng(2)
    letters = list(b"abcAB_")
    delims = list(b" \n\t,.'0-") + [0, 0x80, 0xC3, 0xFF]
    alphabet = np.array(letters * 3 + delims, dtype=np.uint8)
    words = ["a", "ab", "abc", "b_a", "A", "aB", "_", "abcabcabcabc", "x" * 31, "ba" * 16]
    for trial in range(400):
        data = _rand_text(rng, int(rng.integers(0, 300)), alphabet)
        for w in words:
            w33 = _word33(w)
            assert oracle.match_string(w33, data) == ref.ref_match_string(w33, data, len(data)), (w, data)
    # a 32-char word against runs of its own letters (the sizecount==32 path)
    w = "ab" * 16
    for k in range(0, 40):
        data = (b"ab" * k)[:k + 20] + b" " + b"ab" * 16 + b" zz"
        w33 = _word33(w)
        assert oracle.match_string(w33, data) == ref.ref_match_string(w33, data, len(data))


def test_fast_equals_faithful(built):
    rng = np.random.default_rng(3)
    vocab = [b"the", b"cat", b"at", b"a", b"zebra", b"x_y", b"Hello", b"q" * 32, b"r" * 31]
    for trial in range(6):
        parts = []
        n = 0
        while n < 70000:
            r = rng.random()
            if r < 0.8:
                t = vocab[int(rng.integers(0, len(vocab)))]
            elif r < 0.9:
                t = b"".join(vocab[int(rng.integers(0, len(vocab)))] for _ in range(int(rng.integers(2, 12))))
            else:
                t = bytes(rng.integers(97, 100, int(rng.integers(30, 80)), dtype=np.uint8))
            parts.append(t)
            parts.append(bytes([int(rng.choice(list(b" \n,.9")))]))
            n += len(t) + 1
        data = b"".join(parts)
        # force a long alpha run across the first window edge at 16384
        data = data[:16370] + b"c" * 60 + data[16430:]
        recs = b"".join(v + b"\0" * (32 - len(v)) for v in vocab + [b"c" * 14, b"cat" + b"\0" + b"zz"])
        f1 = oracle.grep_counts(recs, [data], mode="faithful")
        f2 = oracle.grep_counts(recs, [data], mode="fast", nthreads=1)
        assert np.array_equal(f1, f2), (f1.ravel(), f2.ravel())


def test_split_points(built):
    data = bytearray(b" " * 40000)
    data[16380:16420] = b"k" * 40  # alpha run covering the whole 32-byte halo
    sp = oracle.split_points(bytes(data))
    assert list(sp) == [16384 + 32]
    # the run is cut at 16416: the reference counts its 4-char tail as a token
    rec = b"kkkk" + b"\0" * 28
    assert oracle.grep_counts(rec, [bytes(data)], mode="faithful")[0, 0] == 1
    assert oracle.grep_counts(rec, [bytes(data)], mode="fast")[0, 0] == 1


def test_duplicate_and_empty_records(built):
    data = b"dog cat dog\n"
    recs = (b"dog" + b"\0" * 29) + (b"\0" * 32) + (b"dog" + b"\0" * 29) + (b"cat\0junk" + b"\0" * 24)
    for mode in ("fast", "faithful", "refalgo"):
        c = oracle.grep_counts(recs, [data], mode=mode).ravel().tolist()
        assert c == [2, 0, 2, 1], (mode, c)


def test_gemv_f64(built):
    rng = np.random.default_rng(4)
    A = rng.standard_normal((37, 129)).astype(np.float32)
    x = rng.standard_normal(129).astype(np.float32)
    y, ay = oracle.gemv_f64(A, x)
    want = A.astype(np.float64) @ x.astype(np.float64)
    assert np.allclose(y, want, rtol=1e-12, atol=1e-12)
    assert np.allclose(ay, np.abs(A.astype(np.float64) * x.astype(np.float64)).sum(1))


def test_reference_fixture_counts(built):
    """The reference's own inputs (dict.gpu x pg100.txt.small): the fast
    oracle equals the faithful walk whose matcher is pinned to the reference
    code; the digest is committed so the result cannot drift."""
    root = oracle.reference_root()
    d = os.path.join(root, "samples/grep_text/input/dict.gpu")
    t = os.path.join(root, "samples/grep_text/input/pg100.txt.small")
    if not (os.path.exists(d) and os.path.exists(t)):
        pytest.skip("reference inputs not on this machine")
    recs = open(d, "rb").read()[:32 * 4000]
    text = open(t, "rb").read()
    fast = oracle.grep_counts(recs, [text], mode="fast")
    faith = oracle.grep_counts(recs, [text], mode="faithful")
    assert np.array_equal(fast, faith)
    with open(os.path.join(GOLDEN, "reference_fixture_counts.json")) as f:
        g = json.load(f)
    assert int(fast.sum()) == g["total"]
    assert oracle.xxh64(fast.astype("<u4").tobytes()) == int(g["xxh64"], 16)


def test_reference_cpu_path_equals_faithful(built):
    """The reference's own match_string, driven through its window walk,
    equals the faithful restatement (also on long runs across windows)."""
    rng = np.random.default_rng(11)
    words = [b"cat", b"at", b"kkkk", b"k" * 32, b"tail"]
    recs = b"".join(w + b"\0" * (32 - len(w)) for w in words)
    data = bytearray(rng.choice(list(b"catk \n."), 60000).astype(np.uint8).tobytes())
    data[16370:16450] = b"k" * 76 + b"tail"
    got = oracle.ref_grep_counts(recs, [bytes(data), bytes(data[:30000])], nthreads=2)
    if got is None:
        pytest.skip("reference matcher not built")
    want = oracle.grep_counts(recs, [bytes(data), bytes(data[:30000])], mode="faithful")
    assert np.array_equal(got, want)

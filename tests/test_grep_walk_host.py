"""The host walk that grep plans run over every file at open (CPU only: no
CUDA call is made).  It finds the bytes the reference's chunk walk reads a
second time (samples/grep_text/grep_text_gpu.cu:298-318: the cursor moves
16384 bytes after the last window too, so a last window longer than 16384
bytes is followed by one more of the bytes past it), whose tokens
k_grep_tail then counts again.  It must agree with the oracle's own
restatement of that walk on every input."""
import ctypes

import numpy as np

import gpufs_gb300
from oracle import oracle

W = 16384


def _lib():
    lib = ctypes.CDLL(gpufs_gb300.LIB_PATH)
    lib.gfs__grep_tail_start.restype = ctypes.c_uint64
    lib.gfs__grep_tail_start.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
    return lib


def _product(lib, b):
    a = np.frombuffer(b, dtype=np.uint8)
    return int(lib.gfs__grep_tail_start(a.ctypes.data if a.size else None, a.size))


def _cursors(b):
    """Cursors of the reference walk over b, for building cases."""
    c, out = 0, [0]
    while len(b) - c >= W + 32:
        ov = 0
        while ov < 32 and (chr(b[c + W + ov]).isalpha() and b[c + W + ov] < 128 or b[c + W + ov] == 95):
            ov += 1
        c += W + ov
        out.append(c)
    return out


def test_sizes_around_one_window(built):
    lib = _lib()
    for n in [0, 1, 31, W - 1, W, W + 1, W + 17, W + 31, W + 32, W + 33, 2 * W, 2 * W + 5, 3 * W + 40]:
        for fill in (b" ", b"a", b"ab c"):
            b = (fill * (n // len(fill) + 1))[:n]
            assert _product(lib, b) == oracle.tail_start(b), (n, fill)
    # one window longer than 16384 bytes: the bytes past 16384 are read twice
    assert _product(lib, b" " * (W + 5)) == W
    assert _product(lib, b" " * W) == W
    assert _product(lib, b"") == 0


def test_tails_after_drifting_windows(built):
    """Files cut so that the walk's last window is 16385..16415 bytes long,
    after windows whose halos began with letters (the cursor drifts)."""
    lib = _lib()
    rng = np.random.default_rng(21)
    alph = np.array(list(b"abAB_x") * 4 + list(b" \n.9") + [0, 200], dtype=np.uint8)
    found = 0
    for trial in range(300):
        big = rng.choice(alph, 120000).astype(np.uint8)
        if trial % 2:
            k = int(rng.integers(0, 110000))
            big[k:k + int(rng.integers(30, 90))] = ord("a")
        b = big.tobytes()
        cs = _cursors(b)
        k = int(rng.integers(0, len(cs) - 1))
        cut = cs[k] + W + int(rng.integers(1, 32))
        got = _product(lib, b[:cut])
        assert got == oracle.tail_start(b[:cut]) == cs[k] + W, (trial, cut)
        found += 1
        # and a random cut, mostly with no such bytes
        cut = int(rng.integers(0, len(b)))
        assert _product(lib, b[:cut]) == oracle.tail_start(b[:cut]), (trial, cut)
    assert found == 300


def test_tail_counts_are_what_the_reference_adds(built):
    """Hand cases: the reference counts the tokens past 16384 twice (a word
    cut by the second window's start counts as its piece)."""
    lib = _lib()
    words = [b"aaaa", b"bb", b"aaaaaaaa"]
    recs = b"".join(w + b"\0" * (32 - len(w)) for w in words)
    cases = [(b" " * W + b"aaaa", [2, 0, 0]),
             (b" " * W + b"aaaa bb", [2, 2, 0]),
             (b" " * (W - 4) + b"aaaaaaaa bb", [1, 2, 1])]
    for text, want in cases:
        assert _product(lib, text) == W
        for mode in ("fast", "faithful", "refalgo"):
            assert oracle.grep_counts(recs, [text], mode=mode).ravel().tolist() == want, mode
        ref = oracle.ref_grep_counts(recs, [text], nthreads=1)
        if ref is not None:
            assert ref.ravel().tolist() == want


try:
    from hypothesis import given, settings, strategies as st
except ImportError:  # the cases above still run
    given = None

if given is not None:
    @settings(max_examples=200, deadline=None)
    @given(body=st.lists(st.sampled_from(list(b"ab_A ") + [0, 250]), min_size=0, max_size=300).map(bytes),
           shift=st.integers(min_value=0, max_value=3 * W + 200))
    def test_walk_agrees_with_oracle(built, body, shift):
        lib = _lib()
        b = (b"a b " * (shift // 4 + 1))[:shift] + body
        assert _product(lib, b) == oracle.tail_start(b)

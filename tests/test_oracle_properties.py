"""Property tests of the grep oracle (CPU only; skipped where hypothesis is
absent): on arbitrary dictionaries and texts, the single-pass matcher, the
faithful restatement of the reference's window walk and the reference's
per-word algorithm give the same counts, and, where the reference-derived
library is built, so does the reference's own match_string driven through
its window walk (samples/grep_text/grep_text_gpu.cu:139-160,193-387)."""
import numpy as np
import pytest

from oracle import oracle

hyp = pytest.importorskip("hypothesis")
st = pytest.importorskip("hypothesis.strategies")
from hypothesis import HealthCheck, given, settings  # noqa: E402

# letters of both cases and '_' (the reference's alpha), digits and
# punctuation that delimit, NUL, and bytes above 0x7F (signed as char)
TEXT_BYTES = list(b"abAB_") * 3 + list(b" \n9'-.") + [0, 0x80, 0xC3, 0xFF]
WORD_BYTES = list(b"abAB_")
WINDOW = 16384  # grep_text_gpu.cu:302-306: a 16 KiB window plus a 32-byte halo

words = st.lists(
    st.one_of(
        st.binary(min_size=0, max_size=0),                                      # empty record
        st.lists(st.sampled_from(WORD_BYTES), min_size=1, max_size=6).map(bytes),
        st.lists(st.sampled_from(WORD_BYTES), min_size=28, max_size=32).map(bytes),
        # records with bytes that are not letters: no token can equal them
        st.lists(st.sampled_from(WORD_BYTES + list(b"9' -") + [0x80, 0xFF]), min_size=1, max_size=8).map(bytes),
        st.tuples(st.lists(st.sampled_from(WORD_BYTES), min_size=1, max_size=5).map(bytes),
                  st.binary(min_size=1, max_size=8)).map(lambda t: (t[0] + b"\0" + t[1])[:32]),
    ),
    min_size=1, max_size=12)

texts = st.lists(st.sampled_from(TEXT_BYTES), min_size=0, max_size=400).map(bytes)


def _records(ws):
    return b"".join(w[:32] + b"\0" * (32 - len(w[:32])) for w in ws)


def _all_modes(recs, files):
    fast = oracle.grep_counts(recs, files, mode="fast", nthreads=1)
    faithful = oracle.grep_counts(recs, files, mode="faithful")
    refalgo = oracle.grep_counts(recs, files, mode="refalgo", nthreads=1)
    assert np.array_equal(fast, faithful), (fast.ravel(), faithful.ravel())
    assert np.array_equal(refalgo, faithful), (refalgo.ravel(), faithful.ravel())
    ref = oracle.ref_grep_counts(recs, files, nthreads=1)
    if ref is not None:
        assert np.array_equal(ref, faithful), (ref.ravel(), faithful.ravel())


@settings(max_examples=150, deadline=None, suppress_health_check=[HealthCheck.too_slow])
@given(ws=words, files=st.lists(texts, min_size=1, max_size=3))
def test_modes_agree_on_short_texts(built, ws, files):
    _all_modes(_records(ws), files)


@settings(max_examples=40, deadline=None, suppress_health_check=[HealthCheck.too_slow])
@given(ws=words, tail=texts, shift=st.integers(min_value=-40, max_value=40),
       run=st.integers(min_value=0, max_value=70))
def test_modes_agree_across_a_window_edge(built, ws, tail, shift, run):
    """A token or a long letter run placed across the first window edge,
    where the reference cuts runs of 33 or more letters."""
    head = b" " * (WINDOW + shift) + b"a" * run
    _all_modes(_records(ws + [b"a" * 4, b"a" * 32]), [head + tail])

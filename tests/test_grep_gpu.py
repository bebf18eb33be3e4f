"""grep_text on the GPU equals the oracle (the reference's match_string
semantics, including its chunk-walk cuts of long letter runs)."""
import os

import numpy as np
import pytest

import gpufs_gb300 as g
from gpufs_gb300 import datagen
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sess(built):
    s = g.Session(log_page=16, pool_bytes=512 << 20, max_files=256, timeout_s=20)
    yield s
    s.close()


def _check(sess, dpath, paths, n_ctas=0, direct=False):
    with g.Grep(sess, dpath, paths) as gr:
        gr.run(n_ctas, direct=direct)  # direct: mapped files read by the GPU, bypassing the cache
        got = gr.counts()
        gr.run(n_ctas)  # cached run (the second one cache-resident): same answer
        got2 = gr.counts()
    want = oracle.grep_counts(open(dpath, "rb").read(), [open(p, "rb").read() for p in paths], mode="fast")
    assert got.shape == want.shape
    bad = np.argwhere(got != want)
    assert bad.size == 0, (bad[:5], got[tuple(bad[0])], want[tuple(bad[0])])
    assert np.array_equal(got, got2)
    return got


def test_zipf_corpus(sess, shm_dir):
    paths, dpath = datagen.grep_corpus(shm_dir, n_files=5, total_bytes=9 * (1 << 20) + 12345, n_vocab=5000,
                                       n_dict=2000, seed=3)
    got = _check(sess, dpath, paths)
    assert got.sum() > 100000
    assert sess.last_error() == 0


@pytest.mark.parametrize("n_ctas", [1, 7, 152, 600])
def test_grid_sizes(sess, shm_dir, n_ctas):
    paths, dpath = datagen.grep_corpus(shm_dir, n_files=3, total_bytes=3 * (1 << 20) + 777, n_vocab=3000,
                                       n_dict=1000, seed=4)
    _check(sess, dpath, paths, n_ctas)


def _write(path, data):
    with open(path, "wb") as f:
        f.write(data)


def test_adversarial_tokens(sess, shm_dir):
    """Upper case, underscores, digits, bytes >= 0x80, NULs, tokens of 31/32/33+
    letters, and long letter runs across the reference's 16384-byte windows."""
    rng = np.random.default_rng(7)
    words = [b"cat", b"Cat", b"c_t", b"_", b"a", b"zz" * 16, b"q" * 31, b"r" * 32, b"tail", b"kkkk", b"ab" * 8]
    recs = b"".join(w + b"\0" * (32 - len(w)) for w in words) + b"\0" * 32 + b"cat" + b"\0" * 29
    dpath = os.path.join(shm_dir, "d.gpu")
    _write(dpath, recs)
    paths = []
    for fi in range(4):
        parts = []
        n = 0
        while n < 150000 + 40000 * fi:
            r = rng.random()
            if r < 0.6:
                t = words[int(rng.integers(0, len(words)))]
            elif r < 0.7:
                t = bytes(rng.integers(0, 256, int(rng.integers(1, 6)), dtype=np.uint8))
            elif r < 0.8:
                t = b"k" * int(rng.integers(30, 70))
            else:
                t = b"".join(words[int(rng.integers(0, 4))] for _ in range(int(rng.integers(1, 4))))
            parts.append(t)
            parts.append(bytes([int(rng.choice(list(b" \n\t.,;09'-\x00\xff")))]))
            n += len(t) + 1
        data = bytearray(b"".join(parts))
        # letter runs crossing window edges (16384, 32768+overlap, ...)
        for base in (16370, 32760, 65530):
            data[base:base + 80] = b"k" * 76 + b"tail"
        p = os.path.join(shm_dir, "adv%d.txt" % fi)
        _write(p, bytes(data))
        paths.append(p)
    assert any(len(oracle.split_points(open(p, "rb").read())) for p in paths)
    _check(sess, dpath, paths)
    _check(sess, dpath, paths, direct=True)


def test_page_sizes_and_tiny_files(built, shm_dir):
    paths, dpath = datagen.grep_corpus(shm_dir, n_files=4, total_bytes=2 * (1 << 20) + 99, n_vocab=2000,
                                       n_dict=500, seed=5)
    t1 = os.path.join(shm_dir, "t1.txt")
    _write(t1, b"")
    t2 = os.path.join(shm_dir, "t2.txt")
    words = open(dpath, "rb").read()
    first = words[:32].rstrip(b"\0")
    _write(t2, first)  # a word right at end of file, no delimiter
    paths = paths + [t1, t2]
    for lp in (12, 14, 16, 20):
        with g.Session(log_page=lp, pool_bytes=128 << 20, timeout_s=20) as s:
            _check(s, dpath, paths, direct=(lp == 14))


def test_large_dictionary_global_table(sess, shm_dir):
    """A dictionary too large for shared memory uses the table in global memory."""
    voc = datagen.vocab(60000, seed=9, minlen=3, maxlen=12)
    dpath = os.path.join(shm_dir, "big.gpu")
    datagen.dictionary(dpath, voc, 58112, seed=2)
    paths = [os.path.join(shm_dir, "z%d.txt" % i) for i in range(2)]
    datagen.zipf_files(paths, [1 << 20, (1 << 20) + 5], voc, s=1.1, seed=8)
    with g.Grep(sess, dpath, paths) as gr:
        assert gr.smem_table == 0
    _check(sess, dpath, paths)


def test_pool_smaller_than_corpus(built, shm_dir):
    paths, dpath = datagen.grep_corpus(shm_dir, n_files=3, total_bytes=24 << 20, n_vocab=3000, n_dict=1000, seed=6)
    with g.Session(log_page=16, pool_bytes=8 << 20, timeout_s=20) as s:
        _check(s, dpath, paths, n_ctas=8)
        assert s.stats()["evictions"] > 0


@pytest.mark.parametrize("n_ctas", [0, 5])
def test_direct_scan_reads_the_mappings(built, shm_dir, n_ctas):
    """The direct scan reads files of 64 KiB and more from their registered
    host mappings (no buffer-cache miss for them) and smaller files through
    the cache; ragged sizes, a file just under and just over the mapping
    threshold, an empty file; counts equal the oracle and a cached run."""
    paths, dpath = datagen.grep_corpus(shm_dir, n_files=5, total_bytes=6 * (1 << 20) + 4321, n_vocab=4000,
                                       n_dict=1500, seed=21)
    text = open(paths[0], "rb").read()
    extra = {"under.txt": text[:65535], "over.txt": text[:65543], "small.txt": text[:5001], "empty.txt": b""}
    for name, data in extra.items():
        p = os.path.join(shm_dir, name)
        _write(p, data)
        paths.append(p)
    want = oracle.grep_counts(open(dpath, "rb").read(), [open(p, "rb").read() for p in paths], mode="fast")
    unmapped_pages = sum((os.path.getsize(p) + 65535) // 65536 for p in paths if os.path.getsize(p) < 65536)
    with g.Session(log_page=16, pool_bytes=256 << 20, timeout_s=20) as s:
        with g.Grep(s, dpath, paths) as gr:
            s.reset_stats()
            gr.run(n_ctas, direct=True)
            got = gr.counts()
            st = s.stats()
            assert 0 < st["misses"] <= unmapped_pages, (st["misses"], unmapped_pages)
            gr.run(n_ctas)
            assert np.array_equal(gr.counts(), got)
        assert s.last_error() == 0
    bad = np.argwhere(got != want)
    assert bad.size == 0, (bad[:5], got[tuple(bad[0])], want[tuple(bad[0])])


def test_large_count_matrix(built, shm_dir):
    """A count matrix over 16 MB (20,000 words x 220 files) comes back in one
    DMA and a multi-threaded host copy, equal to the oracle."""
    voc = datagen.vocab(30000, seed=31)
    dpath = os.path.join(shm_dir, "big.gpu")
    datagen.dictionary(dpath, voc, 20000, seed=32)
    paths = [os.path.join(shm_dir, "m%03d.txt" % i) for i in range(220)]
    datagen.zipf_files(paths, [3000 + 97 * i for i in range(220)], voc, s=1.1, seed=33)
    want = oracle.grep_counts(open(dpath, "rb").read(), [open(p, "rb").read() for p in paths], mode="fast")
    assert want.nbytes > 16 << 20
    with g.Session(log_page=16, pool_bytes=128 << 20, max_files=512, timeout_s=20) as s:
        with g.Grep(s, dpath, paths) as gr:
            gr.run()
            got = gr.counts()
    assert np.array_equal(got, want)


def test_empty_and_degenerate_dictionaries(built, shm_dir):
    """No records, only empty records, and one word repeated: the table
    built on the device handles each, and counts equal the oracle."""
    paths, _ = datagen.grep_corpus(shm_dir, n_files=2, total_bytes=300000, n_vocab=500, n_dict=100, seed=41)
    text = open(paths[0], "rb").read()
    word = text.split()[3][:12]
    cases = {"none.gpu": b"", "empties.gpu": b"\0" * 32 * 5,
             "repeated.gpu": (word + b"\0" * (32 - len(word))) * 7 + b"\0" * 32}
    with g.Session(log_page=16, pool_bytes=64 << 20, timeout_s=20) as s:
        for name, recs in cases.items():
            dpath = os.path.join(shm_dir, name)
            _write(dpath, recs)
            want = oracle.grep_counts(recs, [open(p, "rb").read() for p in paths], mode="fast")
            got = g.grep_text(s, dpath, paths)
            assert got.shape == want.shape and np.array_equal(got, want), name
        assert s.last_error() == 0


def test_one_shot_grep_text(sess, shm_dir):
    paths, dpath = datagen.grep_corpus(shm_dir, n_files=2, total_bytes=1 << 20, n_vocab=1000, n_dict=300, seed=10)
    got = g.grep_text(sess, dpath, paths)
    want = oracle.grep_counts(open(dpath, "rb").read(), [open(p, "rb").read() for p in paths])
    assert np.array_equal(got, want)


def test_many_sessions_in_one_process(built, shm_dir):
    """Sessions created one after another in one process (each with its own
    kernel and worker streams) keep serving cold reads while their kernel
    occupies every SM."""
    paths, dpath = datagen.grep_corpus(shm_dir, n_files=4, total_bytes=2 * (1 << 20) + 99, n_vocab=2000,
                                       n_dict=500, seed=12)
    want = oracle.grep_counts(open(dpath, "rb").read(), [open(p, "rb").read() for p in paths])
    for i in range(12):
        with g.Session(log_page=(12, 14, 16)[i % 3], pool_bytes=64 << 20, host_workers=8 + (i % 3) * 4,
                       timeout_s=10) as s:
            with g.Grep(s, dpath, paths) as gr:
                gr.run(0)
                assert np.array_equal(gr.counts(), want), i


def _batch_files(d, seed):
    """Files of uneven sizes, half Zipf text, half random bytes; sizes around
    the batched chunk (15,360 B), a 32-byte stripe and pages, plus empties."""
    rng = np.random.default_rng(seed)
    voc = datagen.vocab(3000, seed=seed)
    sizes = [0, 1, 31, 32, 33, 63, 4096, 15359, 15360, 15361, 30720, 65537, 100000, 1 << 20,
             3 * (1 << 20) + 7, 0, 5]
    sizes += [int(x) for x in rng.integers(1, 400000, 16)]
    paths = []
    for i, n in enumerate(sizes):
        p = os.path.join(d, "b%03d.dat" % i)
        if i % 2:
            datagen.uniform_bytes(p, n, seed=seed * 100 + i)
        else:
            datagen.zipf_files([p], [n], voc, s=1.1, seed=seed * 100 + i)
        paths.append(p)
    dpath = os.path.join(d, "bdict.gpu")
    datagen.dictionary(dpath, voc, 900, seed=seed)
    return paths, dpath


@pytest.mark.parametrize("n_ctas,pool_mb", [(0, 512), (5, 6)])
def test_batched_counts_and_xxh64(built, shm_dir, n_ctas, pool_mb):
    """The batched form (whole files per CTA, longest first, one graph) gives
    every file's counts and XXH64 exactly; replays agree; a pool smaller
    than the files forces eviction."""
    paths, dpath = _batch_files(shm_dir, seed=11 + pool_mb)
    files = [open(p, "rb").read() for p in paths]
    want = oracle.grep_counts(open(dpath, "rb").read(), files, mode="fast")
    want_x = oracle.xxh64_many([np.frombuffer(f, dtype=np.uint8) for f in files])
    with g.Session(log_page=16, pool_bytes=pool_mb << 20, max_files=256, timeout_s=30) as s:
        with g.Grep(s, dpath, paths) as gr:
            xxh, _ = gr.batch(n_ctas)
            got = gr.counts()
            assert xxh == want_x
            bad = np.argwhere(got != want)
            assert bad.size == 0, (bad[:5], got[tuple(bad[0])], want[tuple(bad[0])])
            xxh2, _ = gr.batch(n_ctas)  # graph replay
            assert xxh2 == want_x and np.array_equal(gr.counts(), want)
            gr.run(n_ctas)  # the plain scan agrees
            assert np.array_equal(gr.counts(), want)
        if pool_mb < 8:
            assert s.stats()["evictions"] > 0
        assert s.last_error() == 0


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("host_table", [False, True])
def test_reference_fixture_inputs(built, host_table):
    """The reference's own grep inputs (the first 4000 records of
    samples/grep_text/input/dict.gpu over samples/grep_text/input/pg100.txt.small,
    copied into tests/golden by make_golden.py): the cold, resident and
    direct scans give the committed digest of the oracle pinned to the
    reference's match_string."""
    import json
    dpath = os.path.join(GOLDEN, "ref_dict_4000.gpu")
    tpath = os.path.join(GOLDEN, "ref_pg100_small.txt")
    with open(os.path.join(GOLDEN, "reference_fixture_counts.json")) as f:
        want = json.load(f)
    for lp in (12, 16):
        with g.Session(log_page=lp, pool_bytes=64 << 20, timeout_s=20, host_table=host_table) as s:
            with g.Grep(s, dpath, [tpath]) as gr:
                for direct in (False, False, True):
                    gr.run(0, direct=direct)
                    got = gr.counts()
                    assert int(got.sum()) == want["total"]
                    assert oracle.xxh64(got.astype("<u4").tobytes()) == int(want["xxh64"], 16)
            assert s.last_error() == 0


def test_host_built_table(built, shm_dir):
    """The host build of the dictionary table (the device build's fallback,
    forced here) gives the same counts as the oracle, for short and long
    words, duplicates and an empty record."""
    paths, dpath = datagen.grep_corpus(shm_dir, n_files=3, total_bytes=3 * (1 << 20) + 5, n_vocab=6000,
                                       n_dict=3000, seed=51)
    recs = open(dpath, "rb").read()
    extra = [b"x" * 17, b"y" * 24, b"z" * 32, recs[:32].rstrip(b"\0"), b""]
    recs += b"".join(w + b"\0" * (32 - len(w)) for w in extra)
    d2 = os.path.join(shm_dir, "hdict.gpu")
    _write(d2, recs)
    with open(paths[0], "ab") as f:
        f.write(b" " + b"x" * 17 + b" " + b"y" * 24 + b"\n" + b"z" * 32 + b" " + b"y" * 25 + b" ")
    with g.Session(log_page=16, pool_bytes=128 << 20, timeout_s=20, host_table=True) as s:
        _check(s, d2, paths)
        _check(s, d2, paths, direct=True)
        assert s.last_error() == 0


def test_table_seeds_and_sizes(built, shm_dir):
    """Dictionaries of 1, 2, 33 and 5000 words: the device-built table gives
    the oracle's counts."""
    voc = datagen.vocab(8000, seed=61)
    paths = [os.path.join(shm_dir, "s%d.txt" % i) for i in range(2)]
    datagen.zipf_files(paths, [400000, 123457], voc, s=1.1, seed=62)
    texts = [open(p, "rb").read() for p in paths]
    with g.Session(log_page=16, pool_bytes=64 << 20, timeout_s=20) as s:
        for nd in (1, 2, 33, 5000):
            dpath = os.path.join(shm_dir, "sd%d.gpu" % nd)
            datagen.dictionary(dpath, voc, nd, seed=63 + nd)
            want = oracle.grep_counts(open(dpath, "rb").read(), texts, mode="fast")
            got = g.grep_text(s, dpath, paths)
            assert np.array_equal(got, want), nd
        assert s.last_error() == 0


@pytest.mark.parametrize("shift", [0, 4, 8, 12])
def test_counts_into_any_host_buffer(sess, shm_dir, shift):
    """The counts reach the caller's buffer whatever its alignment (the
    device writes it with 16-byte stores where the address allows, else
    4-byte ones), and the one-call grep_text's merged run + counts gives the
    same matrix."""
    paths, dpath = datagen.grep_corpus(shm_dir, n_files=3, total_bytes=2 * (1 << 20) + 4321, n_vocab=3000,
                                       n_dict=777, seed=11)
    with g.Grep(sess, dpath, paths) as gr:
        gr.run(0, direct=True)
        want = gr.counts()
        n = want.size
        raw = np.full(n * 4 + 64, 0xAB, dtype=np.uint8)
        base = (-raw.ctypes.data) % 16 + shift  # 16-byte aligned plus shift
        view = raw[base:base + n * 4].view(np.uint32)
        assert sess.L.gfs_grep_counts(gr._h, view.ctypes.data) == 0
        assert np.array_equal(view.reshape(want.shape), want)
        assert np.all(raw[:base] == 0xAB) and np.all(raw[base + n * 4:] == 0xAB)  # nothing outside written
    assert np.array_equal(g.grep_text(sess, dpath, paths), want)


def _walk_cursors(b):
    """Cursors of the reference's chunk walk over b (windows of 16384 + 32
    bytes; a window short of the end moves on by 16384 plus the letters that
    begin its halo)."""
    alpha = set(range(65, 91)) | set(range(97, 123)) | {95}
    c, out = 0, [0]
    while len(b) - c >= 16416:
        ov = 0
        while ov < 32 and b[c + 16384 + ov] in alpha:
            ov += 1
        c += 16384 + ov
        out.append(c)
    return out


def test_bytes_the_reference_reads_twice(sess, shm_dir):
    """When the reference's last window is longer than 16384 bytes its walk
    goes round once more and counts the tokens past 16384 a second time
    (grep_text_gpu.cu:298-318).  Files cut so, small (read with pread) and
    large (read through their mappings, after windows whose halos began with
    letters), give the oracle's counts in every form: cached, direct,
    batched and one call."""
    voc = datagen.vocab(300, seed=71, minlen=2, maxlen=5)
    dpath = os.path.join(shm_dir, "dict.gpu")
    datagen.dictionary(dpath, voc, 300, seed=72)
    raw = open(dpath, "rb").read()
    words = [raw[i:i + 32].rstrip(b"\0") for i in range(0, len(raw), 32)]
    words = [w for w in words if w and b"\0" not in w]
    big = os.path.join(shm_dir, "z.txt")
    datagen.zipf_files([big], [600000], voc, s=1.1, seed=73)
    z = open(big, "rb").read()
    cs = _walk_cursors(z)
    texts = [b" " * 16384 + words[0] + b" " + words[1],                    # one window of 16384 + a few
             b"x" * 16380 + words[2] + b"." + words[0]]                      # a word cut by the second read
    for k in (5, 17, len(cs) - 3):                                            # mapped files (> 64 KiB)
        for d in range(31, 0, -1):
            t = z[:cs[k] + 16384 + d]
            if oracle.tail_start(t) < len(t) and any(w in t[cs[k] + 16384:] for w in words):
                texts.append(t)
                break
    texts.append(z)
    paths = []
    for i, t in enumerate(texts):
        p = os.path.join(shm_dir, "t%d.txt" % i)
        _write(p, t)
        paths.append(p)
    assert sum(oracle.tail_start(t) < len(t) for t in texts) >= 4
    want = oracle.grep_counts(raw, texts, mode="fast")
    for i, t in enumerate(texts):
        if len(t) < 100000:
            assert np.array_equal(want[:, i], oracle.grep_counts(raw, [t], mode="faithful")[:, 0]), i
    with g.Grep(sess, dpath, paths) as gr:
        gr.run(direct=True)
        assert np.array_equal(gr.counts(), want)
        gr.run()
        assert np.array_equal(gr.counts(), want)
        gr.batch()
        assert np.array_equal(gr.counts(), want)
    assert np.array_equal(g.grep_text(sess, dpath, paths), want)
    assert sess.last_error() == 0

/*
 * CPU oracle for the GPU file-system hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it restates, in plain
 * C, what the reference computes on the path, so that the tests, smoke() and
 * the CPU-baseline leg of bench.py can compare the CUDA path against it.  No
 * product code links it; the product fails loudly when its CUDA library is
 * missing instead of falling back here.
 *
 * Pinning (see tests/test_oracle.py):
 *   - orc_xxh64 is written from the public xxHash XXH64 specification and is
 *     checked against the system libxxhash (0.8.x) and its known answers.
 *   - orc_grep_match_string restates the reference's device matcher
 *     (samples/grep_text/grep_text_gpu.cu:79 `alpha`, :139-160 `match_string`)
 *     and is checked byte-for-byte against that very function compiled from
 *     the reference source into oracle/_ref/ (oracle/build_ref.sh).
 *   - orc_grep_file_faithful restates the reference's per-file chunk loop
 *     (grep_text_gpu.cu:89-101 `find_overlap`, :298-329) around match_string.
 *   - orc_grep_counts_fast is the single-pass restatement (tokenise once, hash
 *     lookup, plus the walk's cut points and the tail it reads twice:
 *     orc_grep_split_points, orc_grep_tail_start); it is checked against
 *     orc_grep_file_faithful on random, adversarial and property-generated
 *     inputs.
 *   - orc_gemv_f64 is the FP64 host GEMV the bigmatrix sample is checked against
 *     (samples/bigmatrix_mmap/bigmatrix_mmap.cu:24-41 computes the FP32 dot).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

/* ------------------------------------------------------------------------- */
/* XXH64, from the published xxHash specification (XXH64 algorithm).          */
/* ------------------------------------------------------------------------- */
#define P64_1 0x9E3779B185EBCA87ULL
#define P64_2 0xC2B2AE3D27D4EB4FULL
#define P64_3 0x165667B19E3779F9ULL
#define P64_4 0x85EBCA77C2B2AE63ULL
#define P64_5 0x27D4EB2F165667C5ULL

static inline uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
static inline uint64_t rd64(const uint8_t* p) {
    uint64_t v = 0;
    for (int i = 7; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}
static inline uint32_t rd32(const uint8_t* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
static inline uint64_t xround(uint64_t acc, uint64_t in) {
    acc += in * P64_2;
    acc = rotl64(acc, 31);
    return acc * P64_1;
}
static inline uint64_t xmerge(uint64_t acc, uint64_t v) {
    acc ^= xround(0, v);
    return acc * P64_1 + P64_4;
}

uint64_t orc_xxh64(const void* data, size_t len, uint64_t seed) {
    const uint8_t* p = (const uint8_t*)data;
    const uint8_t* end = p + len;
    uint64_t h;
    if (len >= 32) {
        uint64_t v1 = seed + P64_1 + P64_2, v2 = seed + P64_2, v3 = seed, v4 = seed - P64_1;
        const uint8_t* limit = end - 32;
        do {
            v1 = xround(v1, rd64(p));
            v2 = xround(v2, rd64(p + 8));
            v3 = xround(v3, rd64(p + 16));
            v4 = xround(v4, rd64(p + 24));
            p += 32;
        } while (p <= limit);
        h = rotl64(v1, 1) + rotl64(v2, 7) + rotl64(v3, 12) + rotl64(v4, 18);
        h = xmerge(h, v1);
        h = xmerge(h, v2);
        h = xmerge(h, v3);
        h = xmerge(h, v4);
    } else {
        h = seed + P64_5;
    }
    h += (uint64_t)len;
    while (p + 8 <= end) {
        h ^= xround(0, rd64(p));
        h = rotl64(h, 27) * P64_1 + P64_4;
        p += 8;
    }
    if (p + 4 <= end) {
        h ^= (uint64_t)rd32(p) * P64_1;
        h = rotl64(h, 23) * P64_2 + P64_3;
        p += 4;
    }
    while (p < end) {
        h ^= (uint64_t)(*p) * P64_5;
        h = rotl64(h, 11) * P64_1;
        ++p;
    }
    h ^= h >> 33;
    h *= P64_2;
    h ^= h >> 29;
    h *= P64_3;
    h ^= h >> 32;
    return h;
}

/* ------------------------------------------------------------------------- */
/* grep_text: the reference matcher, restated.                                */
/* ------------------------------------------------------------------------- */

/* grep_text_gpu.cu:79 -- letters and underscore; everything else (digits,
 * apostrophe, whitespace, NUL, bytes >= 0x80) is a delimiter. */
static inline int orc_alpha(unsigned char c) {
    return (c >= 65 && c <= 90) || (c >= 97 && c <= 122) || c == 95;
}

/* grep_text_gpu.cu:139-160.  `word` points at a 33-byte buffer: the 32-byte
 * NUL-padded dictionary record plus one byte.  The reference reads that 33rd
 * byte from uninitialised shared memory (prefetch_banks never writes it);
 * here it is taken as NUL.  Returns -1 for an empty word (LEN_ZERO). */
int orc_grep_match_string(const char* word33, const char* data, int data_size) {
    const unsigned char* a = (const unsigned char*)word33;
    const unsigned char* d = (const unsigned char*)data;
    int matches = 0, sizecount = 0, word_start = 1;
    if (a[0] == 0) return -1;
    for (int i = 0; i < data_size; i++) {
        if (!orc_alpha(d[i])) {
            if ((sizecount == 32 || a[sizecount] == 0) && word_start) matches++;
            word_start = 1;
            sizecount = 0;
        } else {
            if (a[sizecount] == d[i]) sizecount++;
            else { word_start = 0; sizecount = 0; }
        }
    }
    return matches;
}

#define REF_CHUNK 16384
#define REF_HALO 32

/* grep_text_gpu.cu:89-101: leading alpha run length at dst, at most 32. */
static int orc_find_overlap(const unsigned char* dst) {
    int i = 0;
    for (; i < 32 && orc_alpha(dst[i]); i++) {}
    return i;
}

/* Faithful per-file count for one dictionary record: the chunk walk of
 * grep_text_gpu.cu:298-329 (16384+32-byte windows, overlap stitching, NUL
 * after the last window).  O(file) per word: small cases only. */
uint32_t orc_grep_file_faithful_word(const char* rec32, const uint8_t* file, size_t size) {
    char word[33];
    memcpy(word, rec32, 32);
    word[32] = 0;
    if (word[0] == 0) return 0;
    unsigned char corpus[REF_CHUNK + REF_HALO + 1];
    uint64_t total = 0;
    size_t cursor = 0;
    while (cursor < size) {
        int last_iter = (size - cursor) < (size_t)(REF_CHUNK + REF_HALO);
        int db_left = last_iter ? (int)(size - cursor) : REF_CHUNK + REF_HALO;
        memcpy(corpus, file + cursor, (size_t)db_left);
        corpus[db_left] = 0;
        int overlap = 0;
        if (!last_iter) {
            overlap = orc_find_overlap(corpus + REF_CHUNK);
            cursor += (size_t)overlap;
        }
        cursor += REF_CHUNK;
        int n = orc_grep_match_string(word, (const char*)corpus,
                                      last_iter ? db_left + 1 : REF_CHUNK + overlap + 1);
        if (n > 0) total += (uint64_t)n;
    }
    return (uint32_t)total;
}

/* counts[w * n_files + f] for every record w and file f (faithful walk). */
void orc_grep_counts_faithful(const uint8_t* dict, int n_words, const uint8_t* const* files,
                              const uint64_t* sizes, int n_files, uint32_t* counts) {
    for (int w = 0; w < n_words; w++)
        for (int f = 0; f < n_files; f++)
            counts[(size_t)w * n_files + f] =
                orc_grep_file_faithful_word((const char*)dict + (size_t)w * 32, files[f], sizes[f]);
}

/* Positions where the reference's chunk walk cuts an alpha run: when the 32
 * bytes after a 16384-byte window are all alpha the window is terminated by
 * the NUL it planted at corpus[16416], and the next window starts inside the
 * run.  Returns the number of cut positions (file offsets of the first byte
 * of the second piece); writes up to `cap` of them. */
size_t orc_grep_split_points(const uint8_t* file, size_t size, uint64_t* out, size_t cap) {
    size_t n = 0, cursor = 0;
    while (cursor < size) {
        if ((size - cursor) < (size_t)(REF_CHUNK + REF_HALO)) break;
        int overlap = orc_find_overlap(file + cursor + REF_CHUNK);
        if (overlap == REF_HALO) {
            if (n < cap) out[n] = cursor + REF_CHUNK + REF_HALO;
            n++;
        }
        cursor += REF_CHUNK + (size_t)overlap;
    }
    return n;
}

/* Start of the bytes the reference's chunk walk reads twice, or `size` when
 * there are none.  The walk moves its cursor by 16384 after its last window
 * too (grep_text_gpu.cu:318: `_cursor += CORPUS_PREFETCH_SIZE` whatever
 * last_iter says), so when that window is longer than 16384 bytes the cursor
 * is still inside the file and the loop reads the bytes past it once more, as
 * a window of their own (at most 31 bytes, NUL-terminated like any last
 * window).  Their tokens are counted a second time. */
size_t orc_grep_tail_start(const uint8_t* file, size_t size) {
    size_t cursor = 0;
    while (size - cursor >= (size_t)(REF_CHUNK + REF_HALO))
        cursor += REF_CHUNK + (size_t)orc_find_overlap(file + cursor + REF_CHUNK);
    return size - cursor > (size_t)REF_CHUNK ? cursor + REF_CHUNK : size;
}

/* ------------------------------------------------------------------------- */
/* Single-pass restatement: tokenise once, look each token up.                */
/* ------------------------------------------------------------------------- */
typedef struct {
    uint64_t h;
    int32_t first; /* first record index with this word */
    int32_t used;
} orc_slot;

typedef struct {
    orc_slot* slots;
    uint32_t mask;
    int32_t* next_dup; /* next record with the same word, -1 terminated */
    const uint8_t* dict;
    int n_words;
} orc_dict;

static uint64_t orc_word_hash(const uint8_t* w, int len) {
    uint64_t h = 1469598103934665603ULL;
    for (int i = 0; i < len; i++) { h ^= w[i]; h *= 1099511628211ULL; }
    h ^= (uint64_t)len * P64_5;
    h ^= h >> 31;
    return h;
}

static int rec_len(const uint8_t* rec) {
    int l = 0;
    while (l < 32 && rec[l]) l++;
    return l;
}

static void orc_dict_build(orc_dict* d, const uint8_t* dict, int n_words) {
    uint32_t cap = 16;
    while (cap < (uint32_t)n_words * 2u + 16u) cap <<= 1;
    d->slots = (orc_slot*)calloc(cap, sizeof(orc_slot));
    d->mask = cap - 1;
    d->next_dup = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n_words > 0 ? n_words : 1));
    d->dict = dict;
    d->n_words = n_words;
    for (int w = 0; w < n_words; w++) {
        d->next_dup[w] = -1;
        const uint8_t* rec = dict + (size_t)w * 32;
        int len = rec_len(rec);
        if (len == 0) continue;
        uint64_t h = orc_word_hash(rec, len);
        uint32_t i = (uint32_t)h & d->mask;
        for (;;) {
            orc_slot* s = &d->slots[i];
            if (!s->used) { s->used = 1; s->h = h; s->first = w; break; }
            const uint8_t* r2 = dict + (size_t)s->first * 32;
            if (s->h == h && rec_len(r2) == len && memcmp(r2, rec, (size_t)len) == 0) {
                int t = s->first;
                while (d->next_dup[t] >= 0) t = d->next_dup[t];
                d->next_dup[t] = w;
                break;
            }
            i = (i + 1) & d->mask;
        }
    }
}

static void orc_dict_free(orc_dict* d) { free(d->slots); free(d->next_dup); }

static int orc_dict_find(const orc_dict* d, const uint8_t* tok, int len) {
    uint64_t h = orc_word_hash(tok, len);
    uint32_t i = (uint32_t)h & d->mask;
    for (;;) {
        const orc_slot* s = &d->slots[i];
        if (!s->used) return -1;
        if (s->h == h) {
            const uint8_t* r = d->dict + (size_t)s->first * 32;
            if (rec_len(r) == len && memcmp(r, tok, (size_t)len) == 0) return s->first;
        }
        i = (i + 1) & d->mask;
    }
}

/* Count one file into column f (stride n_files).  Tokens are maximal alpha
 * runs, additionally cut at the reference's chunk-walk split points. */
static void orc_count_file(const orc_dict* d, const uint8_t* f, size_t n, uint32_t* counts,
                           int n_files, int col) {
    size_t nsplit = orc_grep_split_points(f, n, NULL, 0);
    uint64_t* splits = NULL;
    if (nsplit) {
        splits = (uint64_t*)malloc(sizeof(uint64_t) * nsplit);
        orc_grep_split_points(f, n, splits, nsplit);
    }
    size_t si = 0;
    size_t i = 0;
    while (i < n) {
        if (!orc_alpha(f[i])) { i++; continue; }
        size_t s = i;
        while (i < n && orc_alpha(f[i])) {
            i++;
            while (si < nsplit && splits[si] < i) si++;
            if (si < nsplit && splits[si] == i) break; /* forced cut before byte i */
        }
        size_t len = i - s;
        if (len <= 32) {
            int w = orc_dict_find(d, f + s, (int)len);
            while (w >= 0) {
                counts[(size_t)w * n_files + col] += 1;
                w = d->next_dup[w];
            }
        }
    }
    free(splits);
    /* the bytes the walk reads a second time: their tokens (alpha runs cut
     * at the window's start) count again */
    for (i = orc_grep_tail_start(f, n); i < n;) {
        if (!orc_alpha(f[i])) { i++; continue; }
        size_t s = i;
        while (i < n && orc_alpha(f[i])) i++;
        int w = orc_dict_find(d, f + s, (int)(i - s));
        while (w >= 0) {
            counts[(size_t)w * n_files + col] += 1;
            w = d->next_dup[w];
        }
    }
}

typedef struct {
    const orc_dict* d;
    const uint8_t* const* files;
    const uint64_t* sizes;
    int n_files;
    uint32_t* counts;
    int tid, nthreads;
} orc_grep_job;

static void* orc_grep_worker(void* arg) {
    orc_grep_job* j = (orc_grep_job*)arg;
    for (int f = j->tid; f < j->n_files; f += j->nthreads)
        orc_count_file(j->d, j->files[f], j->sizes[f], j->counts, j->n_files, f);
    return NULL;
}

/* counts[w * n_files + f]; files are split over `nthreads` host threads (one
 * file per thread at a time, so the columns never race). */
void orc_grep_counts_fast(const uint8_t* dict, int n_words, const uint8_t* const* files,
                          const uint64_t* sizes, int n_files, uint32_t* counts, int nthreads) {
    orc_dict d;
    orc_dict_build(&d, dict, n_words);
    memset(counts, 0, sizeof(uint32_t) * (size_t)n_words * (size_t)n_files);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > n_files) nthreads = n_files > 0 ? n_files : 1;
    pthread_t th[256];
    orc_grep_job jobs[256];
    if (nthreads > 256) nthreads = 256;
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = (orc_grep_job){&d, files, sizes, n_files, counts, t, nthreads};
        if (nthreads > 1) pthread_create(&th[t], NULL, orc_grep_worker, &jobs[t]);
    }
    if (nthreads == 1) orc_grep_worker(&jobs[0]);
    else for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    orc_dict_free(&d);
}

/* ------------------------------------------------------------------------- */
/* bigmatrix: FP64 host GEMV over the FP32 inputs.                            */
/* ------------------------------------------------------------------------- */
typedef struct {
    const float* A;
    const float* x;
    long rows, cols;
    double* y;
    double* absy;
    long r0, r1;
} orc_gemv_job;

static void* orc_gemv_worker(void* arg) {
    orc_gemv_job* j = (orc_gemv_job*)arg;
    for (long r = j->r0; r < j->r1; r++) {
        const float* row = j->A + (size_t)r * (size_t)j->cols;
        double s = 0.0, a = 0.0;
        for (long c = 0; c < j->cols; c++) {
            double p = (double)row[c] * (double)j->x[c];
            s += p;
            a += p < 0 ? -p : p;
        }
        j->y[r] = s;
        if (j->absy) j->absy[r] = a;
    }
    return NULL;
}

/* y[r] = sum_c A[r,c] x[c] in FP64; absy[r] = sum_c |A[r,c] x[c]| (the
 * per-element error scale), absy may be NULL. */
void orc_gemv_f64(const float* A, const float* x, long rows, long cols, double* y, double* absy,
                  int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    orc_gemv_job jobs[256];
    long per = (rows + nthreads - 1) / nthreads;
    int started = 0;
    for (int t = 0; t < nthreads; t++) {
        long r0 = t * per, r1 = r0 + per;
        if (r0 >= rows) break;
        if (r1 > rows) r1 = rows;
        jobs[t] = (orc_gemv_job){A, x, rows, cols, y, absy, r0, r1};
        pthread_create(&th[t], NULL, orc_gemv_worker, &jobs[t]);
        started++;
    }
    for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------------- */
/* Reference-algorithm CPU grep (per dictionary word, scan the corpus), used   */
/* as the timed CPU path of the reference: every record rescans every file,    */
/* as grep_text_gpu.cu:322-329 and grep_text_cpu.cpp:120-165 do.              */
/* ------------------------------------------------------------------------- */
typedef struct {
    const uint8_t* dict;
    int n_words;
    const uint8_t* const* files;
    const uint64_t* sizes;
    int n_files;
    uint32_t* counts;
    int tid, nthreads;
} orc_refgrep_job;

static void* orc_refgrep_worker(void* arg) {
    orc_refgrep_job* j = (orc_refgrep_job*)arg;
    for (int w = j->tid; w < j->n_words; w += j->nthreads)
        for (int f = 0; f < j->n_files; f++)
            j->counts[(size_t)w * j->n_files + f] = orc_grep_file_faithful_word(
                (const char*)j->dict + (size_t)w * 32, j->files[f], j->sizes[f]);
    return NULL;
}

void orc_grep_counts_refalgo(const uint8_t* dict, int n_words, const uint8_t* const* files,
                             const uint64_t* sizes, int n_files, uint32_t* counts, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    orc_refgrep_job jobs[256];
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = (orc_refgrep_job){dict, n_words, files, sizes, n_files, counts, t, nthreads};
        pthread_create(&th[t], NULL, orc_refgrep_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

/* XXH64 of many files in parallel (the batched form's checksums). */
typedef struct {
    const uint8_t* const* files;
    const uint64_t* sizes;
    int n;
    uint64_t* out;
    int tid, nthreads;
} orc_xxh_job;

static void* orc_xxh_worker(void* arg) {
    orc_xxh_job* j = (orc_xxh_job*)arg;
    for (int i = j->tid; i < j->n; i += j->nthreads) j->out[i] = orc_xxh64(j->files[i], j->sizes[i], 0);
    return NULL;
}

void orc_xxh64_many(const uint8_t* const* files, const uint64_t* sizes, int n, uint64_t* out,
                    int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    orc_xxh_job jobs[256];
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = (orc_xxh_job){files, sizes, n, out, t, nthreads};
        pthread_create(&th[t], NULL, orc_xxh_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

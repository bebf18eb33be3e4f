/*
 * Seeded synthetic workload generator for the GPU file-system benchmarks.
 *
 * The inputs the reference measures on (a Shakespeare corpus, a word list,
 * random matrices) are replaced by seeded synthetic files with the shapes
 * and value distributions of the workloads: uniform random bytes (memcopy),
 * Zipf(s) text over a random lowercase vocabulary (grep_text), N(0,1) FP32
 * matrices (bigmatrix_mmap), and mixes of the two (batched).
 *
 * Every generator is deterministic for a given seed on any IEEE-754 host:
 * the only floating point used (Zipf weights, Box-Muller) goes through the
 * det_* routines below, which use plain +,-,*,/ in a fixed order (build with
 * -ffp-contract=off), never libm.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <fcntl.h>
#include <unistd.h>

/* ---------------- PRNG: splitmix64 seeding, xoshiro256** streams ---------- */
typedef struct { uint64_t s[4]; } dg_rng;

static uint64_t splitmix64(uint64_t* x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static void rng_seed(dg_rng* r, uint64_t seed, uint64_t stream) {
    uint64_t x = seed ^ (stream * 0xD1342543DE82EF95ULL + 0x2545F4914F6CDD1DULL);
    for (int i = 0; i < 4; i++) r->s[i] = splitmix64(&x);
}
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static inline uint64_t rng_next(dg_rng* r) {
    uint64_t* s = r->s;
    uint64_t res = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t; s[3] = rotl(s[3], 45);
    return res;
}
/* uniform integer in [0, n) (multiply-high, no modulo bias worth noting) */
static inline uint32_t rng_below(dg_rng* r, uint32_t n) {
    return (uint32_t)(((rng_next(r) >> 32) * (uint64_t)n) >> 32);
}
/* uniform double in [0,1) with 53 random bits */
static inline double rng_unit(dg_rng* r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }

/* ---------------- deterministic elementary functions ---------------------- */
static const double LN2_HI = 0.693147180369123816490;
static const double LN2_LO = 1.90821492927058770002e-10;

static double det_log(double x) { /* x > 0, finite */
    int e = 0;
    while (x >= 2.0) { x *= 0.5; e++; }
    while (x < 1.0) { x *= 2.0; e--; }
    if (x > 1.4142135623730951) { x *= 0.5; e++; }
    double z = (x - 1.0) / (x + 1.0), z2 = z * z, term = z, sum = 0.0;
    for (int k = 1; k < 60; k += 2) { sum += term / (double)k; term *= z2; }
    return 2.0 * sum + (double)e * LN2_LO + (double)e * LN2_HI;
}
static double det_exp(double x) {
    double kf = x / 0.69314718055994530942;
    int k = (int)(kf < 0 ? kf - 0.5 : kf + 0.5);
    double r = (x - (double)k * LN2_HI) - (double)k * LN2_LO;
    double term = 1.0, sum = 1.0;
    for (int n = 1; n < 30; n++) { term *= r / (double)n; sum += term; }
    while (k > 0) { sum *= 2.0; k--; }
    while (k < 0) { sum *= 0.5; k++; }
    return sum;
}
static const double DG_PI = 3.14159265358979323846;
static void det_sincos(double t, double* s, double* c) { /* t in [-pi, pi] */
    double t2 = t * t, ts = t, tc = 1.0, ss = 0.0, cs = 0.0;
    for (int n = 0; n < 30; n++) {
        ss += ts; cs += tc;
        ts *= -t2 / (double)((2 * n + 2) * (2 * n + 3));
        tc *= -t2 / (double)((2 * n + 1) * (2 * n + 2));
    }
    *s = ss; *c = cs;
}

/* ---------------- file helpers ------------------------------------------- */
static int write_all(int fd, const void* buf, size_t n, off_t off) {
    const char* p = (const char*)buf;
    while (n) {
        ssize_t w = pwrite(fd, p, n, off);
        if (w <= 0) return -1;
        p += w; n -= (size_t)w; off += w;
    }
    return 0;
}

/* ---------------- uniform bytes ------------------------------------------ */
typedef struct { int fd; uint64_t seed; uint64_t off, len; int err; } ub_job;
#define DG_BLK (1u << 22)

static void* ub_worker(void* a) {
    ub_job* j = (ub_job*)a;
    uint8_t* buf = (uint8_t*)malloc(DG_BLK);
    for (uint64_t o = j->off; o < j->off + j->len; o += DG_BLK) {
        dg_rng r;
        rng_seed(&r, j->seed, o / DG_BLK); /* stream per 4 MiB block: thread-count independent */
        uint64_t n = j->off + j->len - o < DG_BLK ? j->off + j->len - o : DG_BLK;
        for (uint64_t i = 0; i < n; i += 8) {
            uint64_t v = rng_next(&r);
            for (int b = 0; b < 8 && i + (uint64_t)b < n; b++) buf[i + (uint64_t)b] = (uint8_t)(v >> (8 * b));
        }
        if (write_all(j->fd, buf, n, (off_t)o)) { j->err = 1; break; }
    }
    free(buf);
    return NULL;
}

/* Write `nbytes` uniform random bytes to path.  Returns 0 on success. */
int dg_uniform_bytes(const char* path, uint64_t nbytes, uint64_t seed, int nthreads) {
    int fd = open(path, O_CREAT | O_TRUNC | O_WRONLY, 0644);
    if (fd < 0) return -1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 64) nthreads = 64;
    uint64_t nblk = (nbytes + DG_BLK - 1) / DG_BLK;
    uint64_t per = (nblk + (uint64_t)nthreads - 1) / (uint64_t)nthreads * DG_BLK;
    pthread_t th[64];
    ub_job jobs[64];
    int started = 0, err = 0;
    for (int t = 0; t < nthreads; t++) {
        uint64_t off = (uint64_t)t * per;
        if (off >= nbytes) break;
        uint64_t len = nbytes - off < per ? nbytes - off : per;
        jobs[t] = (ub_job){fd, seed, off, len, 0};
        pthread_create(&th[t], NULL, ub_worker, &jobs[t]);
        started++;
    }
    for (int t = 0; t < started; t++) { pthread_join(th[t], NULL); err |= jobs[t].err; }
    if (ftruncate(fd, (off_t)nbytes)) err = 1;
    close(fd);
    return err ? -1 : 0;
}

/* ---------------- vocabulary --------------------------------------------- */
/* n distinct lowercase words, lengths uniform in [minlen, maxlen] (<= 15),
 * written as 16-byte NUL-padded records into out (n * 16 bytes). */
int dg_vocab(uint64_t seed, int n, int minlen, int maxlen, char* out) {
    if (maxlen > 15 || minlen < 1 || maxlen < minlen) return -1;
    uint32_t cap = 1;
    while (cap < (uint32_t)n * 4u) cap <<= 1;
    int32_t* set = (int32_t*)malloc(sizeof(int32_t) * cap);
    for (uint32_t i = 0; i < cap; i++) set[i] = -1;
    dg_rng r;
    rng_seed(&r, seed, 0x766f636162ULL);
    int made = 0;
    long guard = 0;
    while (made < n) {
        if (++guard > (long)n * 1000L) { free(set); return -2; }
        char w[16] = {0};
        int len = minlen + (int)rng_below(&r, (uint32_t)(maxlen - minlen + 1));
        for (int i = 0; i < len; i++) w[i] = (char)('a' + rng_below(&r, 26));
        uint64_t h = 1469598103934665603ULL;
        for (int i = 0; i < len; i++) { h ^= (uint8_t)w[i]; h *= 1099511628211ULL; }
        uint32_t s = (uint32_t)(h ^ (h >> 29)) & (cap - 1);
        int dup = 0;
        while (set[s] >= 0) {
            if (memcmp(out + (size_t)set[s] * 16, w, 16) == 0) { dup = 1; break; }
            s = (s + 1) & (cap - 1);
        }
        if (dup) continue;
        set[s] = made;
        memcpy(out + (size_t)made * 16, w, 16);
        made++;
    }
    free(set);
    return 0;
}

/* ---------------- Zipf sampler (Vose alias over ranks) -------------------- */
typedef struct { uint32_t n; double* prob; uint32_t* alias; } dg_alias;

static void alias_build(dg_alias* a, uint32_t n, double s) {
    double* w = (double*)malloc(sizeof(double) * n);
    double tot = 0;
    for (uint32_t k = 0; k < n; k++) { w[k] = det_exp(-s * det_log((double)(k + 1))); tot += w[k]; }
    a->n = n;
    a->prob = (double*)malloc(sizeof(double) * n);
    a->alias = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* small = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* large = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t ns = 0, nl = 0;
    for (uint32_t k = 0; k < n; k++) {
        w[k] = w[k] * (double)n / tot;
        if (w[k] < 1.0) small[ns++] = k; else large[nl++] = k;
    }
    while (ns && nl) {
        uint32_t l = small[--ns], g = large[--nl];
        a->prob[l] = w[l];
        a->alias[l] = g;
        w[g] = (w[g] + w[l]) - 1.0;
        if (w[g] < 1.0) small[ns++] = g; else large[nl++] = g;
    }
    while (nl) { uint32_t g = large[--nl]; a->prob[g] = 1.0; a->alias[g] = g; }
    while (ns) { uint32_t l = small[--ns]; a->prob[l] = 1.0; a->alias[l] = l; }
    free(small); free(large); free(w);
}
static inline uint32_t alias_draw(const dg_alias* a, dg_rng* r) {
    uint64_t v = rng_next(r);
    uint32_t col = (uint32_t)(((v >> 32) * (uint64_t)a->n) >> 32);
    double u = (double)(v & 0xFFFFFFFFULL) * (1.0 / 4294967296.0);
    return u < a->prob[col] ? col : a->alias[col];
}
static void alias_free(dg_alias* a) { free(a->prob); free(a->alias); }

/* ---------------- Zipf text files ---------------------------------------- */
typedef struct {
    const char* path;
    uint64_t nbytes, seed, stream;
    const char* vocab;
    const dg_alias* zipf;
    int err;
} zt_job;

static int write_zipf_text(const char* path, uint64_t nbytes, uint64_t seed, uint64_t stream,
                           const char* vocab, const dg_alias* zipf) {
    int fd = open(path, O_CREAT | O_TRUNC | O_WRONLY, 0644);
    if (fd < 0) return -1;
    dg_rng r;
    rng_seed(&r, seed, stream);
    const size_t BUF = 1u << 22;
    char* buf = (char*)malloc(BUF + 64);
    size_t fill = 0;
    uint64_t written = 0;
    int line = 0, err = 0;
    while (written + fill < nbytes) {
        uint32_t w = alias_draw(zipf, &r);
        const char* word = vocab + (size_t)w * 16;
        int len = (int)strnlen(word, 16);
        uint64_t left = nbytes - written - fill;
        if ((uint64_t)len + 1 > left) { /* pad the tail with newlines */
            while (written + fill < nbytes) buf[fill++] = '\n';
            break;
        }
        if (line > 0 && line + len + 1 > 80) {
            buf[fill - 1] = '\n'; /* turn the previous separator into a line break */
            line = 0;
        }
        memcpy(buf + fill, word, (size_t)len);
        fill += (size_t)len;
        buf[fill++] = ' ';
        line += len + 1;
        if (fill >= BUF) {
            /* keep the last separator in the buffer: it may become a newline */
            if (write_all(fd, buf, fill - 1, (off_t)written)) { err = 1; break; }
            written += fill - 1;
            buf[0] = buf[fill - 1];
            fill = 1;
        }
    }
    if (!err && fill) {
        buf[fill - 1] = '\n';
        if (write_all(fd, buf, fill, (off_t)written)) err = 1;
    }
    free(buf);
    if (ftruncate(fd, (off_t)nbytes)) err = 1;
    close(fd);
    return err ? -1 : 0;
}

static void* zt_worker(void* a) {
    zt_job* j = (zt_job*)a;
    j->err = write_zipf_text(j->path, j->nbytes, j->seed, j->stream, j->vocab, j->zipf);
    return NULL;
}

/* Write n_files Zipf(s) text files (paths[i], sizes[i]) over the given
 * vocabulary (16-byte records).  Files are independent streams (seed, i). */
int dg_zipf_files(const char* const* paths, const uint64_t* sizes, int n_files, const char* vocab,
                  int n_vocab, double s, uint64_t seed, int nthreads) {
    dg_alias zipf;
    alias_build(&zipf, (uint32_t)n_vocab, s);
    if (nthreads < 1) nthreads = 1;
    int err = 0;
    for (int base = 0; base < n_files; base += nthreads) {
        int cnt = n_files - base < nthreads ? n_files - base : nthreads;
        pthread_t th[256];
        zt_job jobs[256];
        if (cnt > 256) cnt = 256;
        for (int t = 0; t < cnt; t++) {
            jobs[t] = (zt_job){paths[base + t], sizes[base + t], seed, (uint64_t)(base + t), vocab, &zipf, 0};
            pthread_create(&th[t], NULL, zt_worker, &jobs[t]);
        }
        for (int t = 0; t < cnt; t++) { pthread_join(th[t], NULL); err |= jobs[t].err; }
    }
    alias_free(&zipf);
    return err ? -1 : 0;
}

/* Dictionary: n_words vocabulary words sampled without replacement (partial
 * Fisher-Yates), as 32-byte NUL-padded records (the reference's dict.gpu
 * format, grep_text_gpu.cu:221 `total_words=in_size/32`). */
int dg_dictionary(const char* path, const char* vocab, int n_vocab, int n_words, uint64_t seed) {
    if (n_words > n_vocab) return -1;
    uint32_t* idx = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n_vocab);
    for (int i = 0; i < n_vocab; i++) idx[i] = (uint32_t)i;
    dg_rng r;
    rng_seed(&r, seed, 0x64696374ULL);
    for (int i = 0; i < n_words; i++) {
        uint32_t j = (uint32_t)i + rng_below(&r, (uint32_t)(n_vocab - i));
        uint32_t t = idx[i]; idx[i] = idx[j]; idx[j] = t;
    }
    char* out = (char*)calloc((size_t)n_words, 32);
    for (int i = 0; i < n_words; i++) memcpy(out + (size_t)i * 32, vocab + (size_t)idx[i] * 16, 16);
    int fd = open(path, O_CREAT | O_TRUNC | O_WRONLY, 0644);
    int rc = fd < 0 ? -1 : write_all(fd, out, (size_t)n_words * 32, 0);
    if (fd >= 0) close(fd);
    free(out);
    free(idx);
    return rc;
}

/* ---------------- N(0,1) FP32 (Box-Muller) -------------------------------- */
typedef struct { int fd; uint64_t seed, off, count; int err; } nf_job;
#define NF_BLK (1u << 20) /* floats per independent stream */

static void* nf_worker(void* a) {
    nf_job* j = (nf_job*)a;
    float* buf = (float*)malloc(sizeof(float) * NF_BLK);
    for (uint64_t o = j->off; o < j->off + j->count; o += NF_BLK) {
        dg_rng r;
        rng_seed(&r, j->seed, 0x4e4f524dULL + o / NF_BLK);
        uint64_t n = j->off + j->count - o < NF_BLK ? j->off + j->count - o : NF_BLK;
        for (uint64_t i = 0; i < n; i += 2) {
            double u1 = 1.0 - rng_unit(&r); /* (0,1] */
            double u2 = rng_unit(&r);
            double rad = -2.0 * det_log(u1);
            /* sqrt: IEEE correctly rounded */
            double m = __builtin_sqrt(rad);
            double sn, cs;
            det_sincos(2.0 * DG_PI * u2 - DG_PI, &sn, &cs);
            buf[i] = (float)(m * cs);
            if (i + 1 < n) buf[i + 1] = (float)(m * sn);
        }
        if (write_all(j->fd, buf, n * sizeof(float), (off_t)(o * sizeof(float)))) { j->err = 1; break; }
    }
    free(buf);
    return NULL;
}

/* Write `count` N(0,1) floats (little-endian FP32) to path. */
int dg_normal_f32(const char* path, uint64_t count, uint64_t seed, int nthreads) {
    int fd = open(path, O_CREAT | O_TRUNC | O_WRONLY, 0644);
    if (fd < 0) return -1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 64) nthreads = 64;
    uint64_t nblk = (count + NF_BLK - 1) / NF_BLK;
    uint64_t per = (nblk + (uint64_t)nthreads - 1) / (uint64_t)nthreads * NF_BLK;
    pthread_t th[64];
    nf_job jobs[64];
    int started = 0, err = 0;
    for (int t = 0; t < nthreads; t++) {
        uint64_t off = (uint64_t)t * per;
        if (off >= count) break;
        uint64_t n = count - off < per ? count - off : per;
        jobs[t] = (nf_job){fd, seed, off, n, 0};
        pthread_create(&th[t], NULL, nf_worker, &jobs[t]);
        started++;
    }
    for (int t = 0; t < started; t++) { pthread_join(th[t], NULL); err |= jobs[t].err; }
    if (ftruncate(fd, (off_t)(count * sizeof(float)))) err = 1;
    close(fd);
    return err ? -1 : 0;
}

/* ---------------- batched-file sizes ------------------------------------- */
/* n sizes log-uniform in [lo, hi] bytes (seeded), rounded to whole bytes. */
void dg_loguniform_sizes(uint64_t seed, int n, uint64_t lo, uint64_t hi, uint64_t* out) {
    dg_rng r;
    rng_seed(&r, seed, 0x73697a6573ULL);
    double a = det_log((double)lo), b = det_log((double)hi);
    for (int i = 0; i < n; i++) {
        double v = det_exp(a + (b - a) * rng_unit(&r));
        uint64_t s = (uint64_t)v;
        if (s < lo) s = lo;
        if (s > hi) s = hi;
        out[i] = s;
    }
}

/* Deterministic coin per index (the batched form's text/binary mix). */
int dg_coin(uint64_t seed, uint64_t i) {
    uint64_t x = seed ^ (i * 0x9E3779B97F4A7C15ULL);
    return (int)(splitmix64(&x) & 1);
}

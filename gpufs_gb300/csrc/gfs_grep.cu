/*
 * grep_text over the GPU file system: whole-word occurrence counts of every
 * dictionary record in every corpus file, read through the HBM buffer cache.
 *
 * Reference: samples/grep_text/grep_text_gpu.cu:193-387 (kernel grep_text),
 * :139-160 (match_string), :79 (alpha).  The reference gives each thread one
 * dictionary word and rescans every 16 KiB corpus chunk for it -- O(words x
 * corpus bytes).  Here the corpus is read once:
 *
 *   - one persistent 1024-thread CTA per SM owns a contiguous run of
 *     15,872-byte chunks of the concatenated corpus; warp 31 pins the run's
 *     pages in windows (one lane per page, misses in parallel) and streams
 *     chunks from the page frames into a 3-stage shared-memory ring with 1D
 *     TMA bulk copies (cp.async.bulk, mbarrier completion, bounded waits),
 *     asking L2 for the chunks ahead;
 *   - warps 0..30 take (chunk, 512-byte segment) items in order; a segment
 *     is classified with SWAR byte arithmetic (16 bytes per lane), its token
 *     starts compacted into a per-warp list, and each lane then looks up two
 *     tokens per round;
 *   - a token's key (its zero-padded bytes) is hashed and looked up in a
 *     hash-and-displace table in shared memory (gfs_grep_common.h): one
 *     displacement and one 16-bit tag per token; a tag hit is verified
 *     against the 32-byte record and adds to the slot's 32-bit counter;
 *   - counters are flushed to counts[word][file] with global atomics when
 *     the CTA's consumers move to another file.
 *
 * The same kernel, instantiated otherwise, is the one-pass direct scan (each
 * warp loads its segment's window straight from the file's registered host
 * mapping) and the batched scan (CTAs take whole files, a hasher warp adds
 * each file's XXH64).  The served loop (k_serve) runs the segment scanner on
 * requested ranges.  The table is built on the device at open (k_tb_*).
 *
 * Exactness: a token counts for record w iff it equals w (match_string
 * semantics; empty records never match, duplicate records all count).  The
 * reference's chunk walk (grep_text_gpu.cu:298-318) has two more effects,
 * both reproduced, so counts equal the reference on any input:
 *   - it cuts an alpha run when the 32 bytes after a 16384-byte window are
 *     all letters; runs of >= 33 letters are flagged per file and
 *     k_grep_fixup restates the walk for flagged files only;
 *   - a last window longer than 16384 bytes is followed by one more window
 *     of the 1..31 bytes past 16384, whose tokens count again; host threads
 *     find those bytes by the same walk while the first scan runs
 *     (walk_tail_start) and k_grep_tail counts them.
 */
#include <cuda_runtime.h>
#include <cooperative_groups.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <errno.h>
#include <fcntl.h>
#include <unistd.h>
#include <sched.h>
#include <time.h>
#include <sys/mman.h>
#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <string>
#include <thread>
#include <unordered_map>
#include <mutex>
#include <vector>

#include "gfs_device.cuh"
#include "gfs_block.cuh"
#include "gfs_grep_common.h"
#include "gfs_xxh64.cuh"
#include "gfs_runtime.h"
#include "gpufs_gb300.h"

#define GR_CONS 31                    /* consumer warps; warp 31 is the producer */
#define GR_CONS_B 30                  /* batched scan: consumers; warp 30 hashes */
#define GR_THREADS 1024
#define GR_SEG 512                    /* bytes per consumer warp per chunk */
#define GR_CH (GR_CONS * GR_SEG)      /* 15872-byte chunks */
#define GR_CH_B (GR_CONS_B * GR_SEG)  /* 15360-byte chunks of the batched scan */
#define GR_LB 16                      /* look-behind bytes staged before a chunk */
#define GR_LA 64                      /* look-ahead bytes staged after it */
#define GR_STAGE (GR_LB + GR_CH + GR_LA + 32)
#define GR_STAGES 3
#define GR_WIN 32                     /* pages per window, incl. look-behind/ahead */
#define GR_PF 6                       /* chunks prefetched into L2 ahead of their copy */

extern __device__ gfs_state* g_gfs;

struct GrepDev {
    int n_files;
    int n_words;
    const int* fds;
    const uint64_t* sizes;
    const uint64_t* chunk_prefix; /* n_files + 1, in GR_CH chunks */
    uint64_t total_chunks;
    uint32_t m;                   /* table slots */
    uint32_t r;                   /* displacement buckets */
    grep_hashk hk;                /* seeded key-mix multipliers */
    const uint16_t* tags;         /* m slot tags (grep_tag), 0 = empty */
    const uint16_t* disp;         /* r displacements */
    const uint4* rec_lo;          /* m: bytes 0..15 of each slot's record */
    const uint4* rec_hi;          /* m: bytes 16..31 (separate, so the short-word
                                     checks touch half the bytes) */
    const uint32_t* slot_word;    /* first record of each slot, ~0 if empty */
    const int32_t* next_dup;      /* next record with the same word, -1 */
    uint32_t* counts;             /* n_words x n_files */
    uint32_t* long_flags;         /* per file: a run of >= 33 letters was seen */
    uint32_t* status;             /* [0] error bits, [1] first failure: site << 16 | errno */
    uint32_t win_pages;           /* pages per window (two windows per CTA may be pinned) */
    /* batched scan: CTAs take whole files, longest first, and hash them */
    const int* file_order;        /* file indices by decreasing size */
    uint32_t* file_next;          /* next position in file_order */
    unsigned long long* xxh;      /* per-file XXH64 */
    /* direct scan: files with a registered host mapping are read from it by
     * the SMs, bypassing the buffer cache */
    const uint64_t* maps;         /* per file: device address of its host mapping, 0 if none */
    /* per file: where the bytes that the reference's chunk walk reads a
     * second time start (the file size when there are none; k_grep_tail) */
    const uint64_t* tail_start;
};

/* Shared-memory bytes of the table's parts (each a multiple of 128); the
 * plan's global tags and displacements are padded to the same sizes.  The
 * counters have 32 spare entries past the m slots (one per lane; see
 * CountSink::hit_if). */
__host__ __device__ __forceinline__ uint32_t grep_tag_smem(uint32_t m) { return (2u * m + 127u) & ~127u; }
__host__ __device__ __forceinline__ uint32_t grep_disp_smem(uint32_t r) { return (2u * r + 127u) & ~127u; }
__host__ __device__ __forceinline__ uint32_t grep_cnt_smem(uint32_t m) { return (4u * (m + 32u) + 127u) & ~127u; }

namespace {

using namespace gfsd;

/* ---------------- PTX helpers: mbarrier + 1D bulk copy ---------------- */
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
/* try_wait with a suspend-time hint: the thread sleeps in hardware until the
 * phase completes or GR_SUSPEND_NS pass, instead of spinning on the issue
 * slots the scanning warps need */
#define GR_SUSPEND_NS 20000u
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok) : "r"(smem_u32(b)), "r"(parity), "n"(GR_SUSPEND_NS) : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
/* bring bytes into L2 ahead of their copy to shared memory (16-byte aligned
 * address, size a multiple of 16) */
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
template <int NC>
__device__ __forceinline__ void consumers_sync() { asm volatile("bar.sync 1, %0;" ::"r"(NC * 32) : "memory"); }

/* ---------------- byte classification ---------------- */
/* bit 7 of each byte of the result is set iff the byte is [A-Za-z_] */
__device__ __forceinline__ uint32_t alpha4(uint32_t w) {
    uint32_t x = (w | 0x20202020u) & 0x7F7F7F7Fu;       /* fold case, drop bit 7 */
    uint32_t ge = x + 0x1F1F1F1Fu;                       /* bit7: x >= 'a' */
    uint32_t gt = x + 0x05050505u;                       /* bit7: x >  'z' */
    uint32_t u = (w ^ 0x5F5F5F5Fu) & 0x7F7F7F7Fu;        /* '_' -> 0 */
    uint32_t nu = (u + 0x7F7F7F7Fu) | (w ^ 0x5F5F5F5Fu); /* bit7 clear iff '_' */
    return ((ge & ~gt & ~w) | ~nu) & 0x80808080u;
}
/* gather bit 7 of the 4 bytes into bits 0..3 */
__device__ __forceinline__ uint32_t nib4(uint32_t a) { return (a * 0x00204081u) >> 28; }
__device__ __forceinline__ uint32_t alpha16(uint4 v) {
    return nib4(alpha4(v.x)) | (nib4(alpha4(v.y)) << 4) | (nib4(alpha4(v.z)) << 8) | (nib4(alpha4(v.w)) << 12);
}
/* [A-Za-z_]: bit 5 folds upper case onto lower case */
__device__ __forceinline__ uint32_t is_alpha(uint32_t c) {
    return (uint32_t)((c | 32u) - 97u < 26u) | (uint32_t)(c == 95u);
}

/* key of a token of len <= 16 at byte st of a 4-byte aligned smem buffer
 * readable 20 bytes past (st & ~3): five word loads, funnel shifts, and the
 * byte masks of its length from a 17-entry table in shared memory */
__device__ __forceinline__ void key16(const uint8_t* base, uint32_t st, uint32_t len, uint32_t k[4], const uint4* km) {
    const uint32_t* w = (const uint32_t*)(base + (st & ~3u));
    const uint32_t sh = (st & 3u) * 8u;
    const uint32_t x0 = w[0], x1 = w[1], x2 = w[2], x3 = w[3], x4 = w[4];
    const uint4 m = km[len];
    k[0] = __funnelshift_r(x0, x1, sh) & m.x;
    k[1] = __funnelshift_r(x1, x2, sh) & m.y;
    k[2] = __funnelshift_r(x2, x3, sh) & m.z;
    k[3] = __funnelshift_r(x3, x4, sh) & m.w;
}

/* key of any len <= 32 (slow path): 9 word loads */
__device__ __forceinline__ void key32(const uint8_t* base, uint32_t st, uint32_t len, uint32_t k[8]) {
    const uint32_t* w = (const uint32_t*)(base + (st & ~3u));
    const uint32_t sh = (st & 3u) * 8u;
    uint32_t x[9];
#pragma unroll
    for (int i = 0; i < 9; i++) x[i] = w[i];
    const int kb = (int)len * 8;
#pragma unroll
    for (int i = 0; i < 8; i++)
        k[i] = __funnelshift_r(x[i], x[i + 1], sh) & __funnelshift_lc(0xFFFFFFFFu, 0u, (uint32_t)max(kb - 32 * i, 0));
}

__device__ __forceinline__ void flush_slot(const GrepDev& P, uint32_t slot, uint32_t n, int f) {
    uint32_t w = P.slot_word[slot];
    while (w != 0xFFFFFFFFu && (int)w < P.n_words) {
        atomicAdd(&P.counts[(size_t)w * P.n_files + f], n);
        int32_t d = P.next_dup[w];
        w = d < 0 ? 0xFFFFFFFFu : (uint32_t)d;
    }
}

__device__ __forceinline__ bool rec_equal(const GrepDev& P, uint32_t slot, bool rlong, const uint32_t* k, uint32_t len) {
    if (rlong != (len > 16u)) return false;
    const uint4 a = __ldg(P.rec_lo + slot);
    bool eq = a.x == k[0] && a.y == k[1] && a.z == k[2] && a.w == k[3];
    if (eq && rlong) {
        const uint4 b = __ldg(P.rec_hi + slot);
        eq = b.x == k[4] && b.y == k[5] && b.z == k[6] && b.w == k[7];
    }
    return eq;
}

/* The dictionary table a scan works with: slot tags and displacements
 * (shared memory, or the plan's global copy), and (table in shared memory)
 * one 32-bit counter per slot for the current file.  Without shared memory
 * counts go straight to the global count matrix. */
struct Tbl {
    const uint16_t* tags;
    const uint16_t* disp;
    uint32_t* cnt;
};

/* The slot a hash selects: its bucket's displacement, then the slot mix. */
template <bool SMEM>
__device__ __forceinline__ uint32_t tbl_slot(const GrepDev& P, const Tbl& t, uint32_t h) {
    const uint32_t b = grep_bucket(h, P.r);
    const uint32_t d = SMEM ? (uint32_t)t.disp[b] : (uint32_t)__ldg(t.disp + b);
    return grep_slot(h, d, P.m);
}
template <bool SMEM>
__device__ __forceinline__ uint32_t tbl_tag(const Tbl& t, uint32_t slot) {
    return SMEM ? (uint32_t)t.tags[slot] : (uint32_t)__ldg(t.tags + slot);
}

/* A slot counter holds one CTA's count of one word in one file, which the
 * uint32 count matrix bounds anyway: a plain add, no overflow check. */
__device__ __forceinline__ void count_hit(const GrepDev& P, const Tbl& t, bool smem, uint32_t slot, int f) {
    if (smem) atomicAdd(&t.cnt[slot], 1u);
    else flush_slot(P, slot, 1u, f);
}

/* Where a scan's dictionary hits go: the scans count per slot (and flag
 * files with runs of 33+ letters for the fix-up); the served loop counts
 * matching tokens per request. */
struct CountSink {
    const GrepDev& P;
    const Tbl& t;
    bool smem;
    int f;
    __device__ __forceinline__ void hit(uint32_t slot) const { count_hit(P, t, smem, slot, f); }
    /* counts slot if h; with the table in shared memory a miss adds to the
     * lane's own spare counter past the table's m (never flushed), so the
     * add needs no branch */
    __device__ __forceinline__ void hit_if(bool h, uint32_t slot) const {
        if (smem) atomicAdd(&t.cnt[h ? slot : P.m + (threadIdx.x & 31u)], 1u);
        else if (h) flush_slot(P, slot, 1u, f);
    }
    __device__ __forceinline__ void long_run() const { atomicOr(&P.long_flags[f], 1u); }
};
struct TotalSink {
    uint32_t n = 0;
    __device__ __forceinline__ void hit(uint32_t) { n++; }
    __device__ __forceinline__ void hit_if(bool h, uint32_t) { n += h ? 1u : 0u; }
    __device__ __forceinline__ void long_run() {}
};

/* General lookup of a key of any length 1..32: the one slot its hash
 * selects, its tag, then the record. */
template <bool SMEM, class Sink>
__device__ void lookup_hit(const GrepDev& P, const Tbl& t, const uint32_t k[8], uint32_t len, Sink& sink) {
    const uint32_t h = grep_h1(grep_mix(&P.hk, k, (int)len));
    const uint32_t slot = tbl_slot<SMEM>(P, t, h);
    const uint32_t tg = tbl_tag<SMEM>(t, slot);
    if (tg == grep_tag(h, (int)len) && rec_equal(P, slot, (tg & GREP_TAG_LONG) != 0u, k, len)) sink.hit(slot);
}

struct StageDesc {
    uint64_t pos;   /* file offset of chunk byte 0 */
    int f;          /* file; -1 marks the end of a batched CTA's work */
    uint32_t clen;  /* chunk bytes */
    uint32_t avail; /* staged bytes from chunk byte 0 (chunk + look-ahead, to end of file) */
    uint32_t fseq;  /* batched scan: the file's number among this CTA's files */
};

struct Shared {
    uint64_t full[GR_STAGES];
    uint64_t empty[GR_STAGES];
    StageDesc desc[GR_STAGES];
    int frames[2][GR_WIN];
    volatile int abort;
    int err;
    uint32_t win;
    uint32_t next_item; /* consumers take (chunk, segment) items in order */
    uint64_t wait_ns;   /* bound on every mbarrier wait (session timeout) */
    uint4 kmask[17];    /* key byte masks by token length 0..16 */
    int fileseq[8];     /* batched scan: file of fseq j at [j & 7] */
    uint64_t cbar;      /* batched scan: the consumers' flush barrier (bounded waits) */
};

__device__ __forceinline__ void fail(Shared& sh, const GrepDev& P, int e, uint32_t site) {
    sh.err = e;
    sh.abort = 1;
    atomicOr(P.status, e == -GFS_ETIMEDOUT ? GFS_ERRB_TIMEOUT : GFS_ERRB_IO);
    atomicCAS(&P.status[1], 0u, (site << 16) | (uint32_t)(e < 0 ? -e : e));
}

/* Bounded wait on an mbarrier phase by one lane.  false: gave up (abort).
 * Each try suspends for up to GR_SUSPEND_NS; every 16 tries the abort flag
 * and the session's wait limit (%globaltimer) are checked. */
__device__ __forceinline__ bool wait_phase(Shared& sh, const GrepDev& P, uint64_t* bar, uint32_t parity, uint32_t site) {
    uint32_t spins = 0;
    uint64_t t0 = 0;
    while (!mbar_try_wait(bar, parity)) {
        if ((++spins & 15u) == 0u) {
            if (sh.abort) return false;
            const uint64_t now = gtimer();
            if (t0 == 0) t0 = now;
            else if (now - t0 > sh.wait_ns) {
                fail(sh, P, -GFS_ETIMEDOUT, site);
                return false;
            }
        }
    }
    return true;
}

__device__ __forceinline__ int file_of(const GrepDev& P, uint64_t c) {
    int lo = 0, hi = P.n_files - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (P.chunk_prefix[mid] <= c) lo = mid; else hi = mid - 1;
    }
    return lo;
}

/* ---------------- consumer: one 512-byte segment ---------------- */
/* Per-warp scratch: the segment's alpha bitmap (bits 0..511, then the 32
 * bytes after the segment, then a zero word) and the list of token starts. */
#define GR_BM_WORDS 18
#define GR_WSCR (GR_BM_WORDS * 4 + GR_SEG) /* bytes per warp: bitmap + 256 u16 starts */

/* letters from bit r of the bitmap on: 1..32, or 33 for a run of 33+ */
__device__ __forceinline__ uint32_t run_len(const uint32_t* bm, uint32_t r) {
    const uint32_t w = r >> 5, b = r & 31u;
    const uint32_t x = __funnelshift_r(bm[w], bm[w + 1], b);
    if (x != 0xFFFFFFFFu) return (uint32_t)__popc(x & ~(x + 1u)); /* trailing ones */
    return 32u + (__funnelshift_r(bm[w + 1], bm[w + 2], b) & 1u);
}

__device__ __forceinline__ bool key_eq(const uint4 r, const uint32_t k[4]) {
    return r.x == k[0] && r.y == k[1] && r.z == k[2] && r.w == k[3];
}

/* NTOK tokens per lane (list entries tb0 + lane + 32 i), straight-line so
 * their loads overlap, with no branch on the common path.  A token of at
 * most 16 letters: key from five shared words, the short hash (key words
 * 0..3), one displacement and one tag load, on a tag hit the record's
 * first 16 bytes, and one counter add.  Tokens of 17+ letters (rare) take
 * a warp-uniform slow path. */
template <bool SMEM, int NTOK, class Sink>
__device__ __forceinline__ void scan_tokens(const GrepDev& P, const Tbl& tbl, const uint8_t* base, const uint32_t* bm,
                                            const uint16_t* slist, uint32_t seg0, uint32_t tb0, uint32_t n_s,
                                            const uint4* km, Sink& sink) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t st[NTOK], len[NTOK], k[NTOK][4], slot[NTOK];
    bool v[NTOK], c[NTOK];
#pragma unroll
    for (int i = 0; i < NTOK; i++) {
        const uint32_t ti = tb0 + lane + 32u * (uint32_t)i;
        v[i] = ti < n_s;
        st[i] = v[i] ? slist[ti] : seg0;
        /* letters from st on, 1..32 (32 also for longer runs) */
        const uint32_t r = st[i] - seg0, w = r >> 5, b = r & 31u;
        const uint32_t x = __funnelshift_r(bm[w], bm[w + 1], b);
        len[i] = (uint32_t)__popc(x & ~(x + 1u));
    }
#pragma unroll
    for (int i = 0; i < NTOK; i++) key16(base, st[i], len[i] <= 16u ? len[i] : 0u, k[i], km);
#pragma unroll
    for (int i = 0; i < NTOK; i++) {
        const uint32_t a = len[i] * P.hk.c[0] + k[i][0] * P.hk.c[1] + k[i][1] * P.hk.c[2] + k[i][2] * P.hk.c[3] +
                           k[i][3] * P.hk.c[4]; /* grep_mix for len <= 16 */
        const uint32_t h = grep_h1(a);
        slot[i] = tbl_slot<SMEM>(P, tbl, h);
        c[i] = v[i] && len[i] <= 16u && tbl_tag<SMEM>(tbl, slot[i]) == ((h | 1u) & 0x7FFFu); /* grep_tag, len <= 16 */
    }
    uint4 r[NTOK];
#pragma unroll
    for (int i = 0; i < NTOK; i++) r[i] = c[i] ? __ldg(P.rec_lo + slot[i]) : make_uint4(0, 0, 0, 0);
#pragma unroll
    for (int i = 0; i < NTOK; i++) sink.hit_if(c[i] && key_eq(r[i], k[i]), slot[i]);
    /* rare: tokens of 17..32 letters take the general lookup; a run of 33+
     * letters flags the file for the fix-up kernel */
    bool lg = false;
#pragma unroll
    for (int i = 0; i < NTOK; i++) lg |= v[i] && len[i] > 16u;
    if (__any_sync(0xFFFFFFFFu, lg)) {
#pragma unroll
        for (int i = 0; i < NTOK; i++)
            if (v[i] && len[i] > 16u) {
                const uint32_t L = run_len(bm, st[i] - seg0);
                if (L > 32u) sink.long_run();
                else {
                    uint32_t kk[8];
                    key32(base, st[i], L, kk);
                    lookup_hit<SMEM>(P, tbl, kk, L, sink);
                }
            }
    }
}

template <bool SMEM, class Sink>
__device__ __forceinline__ void scan_segment(const GrepDev& P, const Tbl& tbl, const uint8_t* base, const StageDesc& d,
                                             uint32_t segi, uint8_t* wscr, const uint4* km, Sink& sink) {
    const int lane = threadIdx.x & 31;
    uint32_t* bm = (uint32_t*)wscr;
    uint16_t* slist = (uint16_t*)(wscr + GR_BM_WORDS * 4);
    const uint32_t seg0 = segi * GR_SEG;
    const uint32_t clen = d.clen, avail = d.avail;
    if (seg0 >= clen) return;
    const uint32_t off = seg0 + 16u * (uint32_t)lane;
    const uint4 v = *(const uint4*)(base + off);
    /* letters among the staged bytes of this file (< avail); token starts
     * only among the chunk's own bytes (< clen).  Every segment but a file's
     * last has its bytes and the 32 after it staged (and then lies inside
     * the chunk): no masks (a warp-uniform test). */
    uint32_t ax = alpha16(v), a = ax;
    const uint32_t q = seg0 + GR_SEG + (uint32_t)lane;
    uint32_t cont;
    if (__all_sync(0xFFFFFFFFu, seg0 + GR_SEG + 32u <= avail)) {
        cont = __ballot_sync(0xFFFFFFFFu, is_alpha(base[q]));
    } else {
        ax &= off >= avail ? 0u : (avail - off >= 16u ? 0xFFFFu : ((1u << (avail - off)) - 1u));
        a = ax & (off >= clen ? 0u : (clen - off >= 16u ? 0xFFFFu : ((1u << (clen - off)) - 1u)));
        cont = __ballot_sync(0xFFFFFFFFu, q < avail && is_alpha(base[q]));
    }
    /* byte before the segment (the look-behind when seg0 == 0; nothing before
     * the file's first byte) and the 32 bytes after it, one per lane */
    const uint32_t before = (seg0 == 0u && d.pos == 0u) ? 0u : is_alpha(base[(int)seg0 - 1]);
    uint32_t pb = __shfl_up_sync(0xFFFFFFFFu, ax >> 15, 1);
    if (lane == 0) pb = before;
    ((uint16_t*)bm)[lane] = (uint16_t)ax;
    if (lane == 0) {
        bm[16] = cont;
        bm[17] = 0u;
    }
    /* compact the token starts into the list */
    const uint32_t starts = a & ~((a << 1) | pb) & 0xFFFFu;
    const uint32_t cnt = (uint32_t)__popc(starts);
    uint32_t incl = cnt;
#pragma unroll
    for (int dd = 1; dd < 32; dd <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, dd);
        if (lane >= dd) incl += t;
    }
    const uint32_t n_s = __shfl_sync(0xFFFFFFFFu, incl, 31);
    /* a lane's starts into the list: four unrolled predicated steps (16
     * bytes of text rarely hold more tokens), then a warp-uniform loop */
    const uint32_t js = incl - cnt;
    uint32_t mm = starts;
#pragma unroll
    for (uint32_t qq = 0; qq < 4u; qq++) {
        const uint32_t pos = off + (uint32_t)(__ffs(mm) - 1);
        if (mm) slist[js + qq] = (uint16_t)pos;
        mm &= mm - 1u;
    }
    if (__any_sync(0xFFFFFFFFu, mm != 0u))
        for (uint32_t qq = 4u; mm; qq++, mm &= mm - 1u) slist[js + qq] = (uint16_t)(off + (uint32_t)(__ffs(mm) - 1));
    __syncwarp();
    /* rounds of two tokens per lane; a last round of at most 32 tokens takes
     * one per lane (warp-uniform choice) */
    for (uint32_t tb0 = 0; tb0 < n_s; tb0 += 64u) {
        if (n_s - tb0 > 32u) scan_tokens<SMEM, 2>(P, tbl, base, bm, slist, seg0, tb0, n_s, km, sink);
        else scan_tokens<SMEM, 1>(P, tbl, base, bm, slist, seg0, tb0, n_s, km, sink);
    }
}

template <bool SMEM, int NC>
__device__ void flush_counts(const GrepDev& P, const Tbl& t, int f) {
    if constexpr (SMEM) {
        for (uint32_t i = threadIdx.x; i < P.m; i += NC * 32) {
            const uint32_t n = t.cnt[i];
            if (n) {
                t.cnt[i] = 0u;
                flush_slot(P, i, n, f);
            }
        }
    }
}

/* ---------------- producer: pin windows, stream chunks ---------------- */
struct Window {
    uint32_t lb, n;   /* pinned pages [lb, lb + n) */
    int buf;          /* sh.frames[buf] */
    uint32_t last_g;  /* last chunk streamed from it */
    bool live;
};

__device__ int pin_pages(gfs_state* S, Shared& sh, int buf, int fd, uint32_t lb, uint32_t n, bool soft) {
    const int lane = threadIdx.x & 31;
    int r = 0;
    if ((uint32_t)lane < n) {
        PinFile pf = pin_file(S, fd);
        bool fresh;
        r = pin_page(S, pf, lb + (uint32_t)lane, GFS_PIN_READ | (soft ? GFS_PIN_NOALLOC : 0), &fresh);
        if (r >= 0 && fresh) publish_valid(S, (uint32_t)r);
        sh.frames[buf][lane] = r;
    }
    const unsigned bad = __ballot_sync(0xFFFFFFFFu, (uint32_t)lane < n && r < 0 && r != -GFS_ENOMEM);
    const unsigned nomem = __ballot_sync(0xFFFFFFFFu, (uint32_t)lane < n && r == -GFS_ENOMEM);
    if (bad || nomem) {
        if ((uint32_t)lane < n && r >= 0) unpin(S, (uint32_t)r);
        return bad ? __shfl_sync(0xFFFFFFFFu, r, __ffs(bad) - 1) : -GFS_ENOMEM;
    }
    return 0;
}

__device__ void unpin_window(gfs_state* S, Shared& sh, Window& w) {
    const int lane = threadIdx.x & 31;
    if (w.live && (uint32_t)lane < w.n) unpin(S, (uint32_t)sh.frames[w.buf][lane]);
    w.live = false;
}

__device__ void release_window(gfs_state* S, const GrepDev& P, Shared& sh, Window& prev, uint32_t site) {
    const int lane = threadIdx.x & 31;
    if (prev.live) {
        if (lane == 0) wait_phase(sh, P, &sh.full[prev.last_g % GR_STAGES], (prev.last_g / GR_STAGES) & 1u, site);
        __syncwarp();
        unpin_window(S, sh, prev);
    }
}

/* Stream chunks [k, kend) of file f (chunk size CH) into the stage ring,
 * pinning page windows as it goes; g counts the chunks this CTA produced.
 * false: aborted. */
template <uint32_t CH>
__device__ bool stream_file(gfs_state* S, const GrepDev& P, Shared& sh, uint8_t* stages, int f, uint32_t fseq,
                            uint64_t k, uint64_t kend, Window& prev, uint32_t& g) {
    const int lane = threadIdx.x & 31;
    const uint32_t lp = S->log_page, page = S->page_size, pmask = page - 1u;
    /* pages one chunk with its look-behind and look-ahead can touch */
    const uint32_t minwin = (uint32_t)((GR_LB + CH + GR_LA + page - 1) / page) + 1u;
    const uint64_t fsize = P.sizes[f];
    while (k < kend) {
        /* window: chunks [k, kw) whose bytes, look-behind and look-ahead
         * lie in at most sh.win pages */
        const uint64_t lbpos = k * CH >= GR_LB ? k * CH - GR_LB : 0;
        const uint32_t lb = (uint32_t)(lbpos >> lp);
        uint64_t kw;
        uint32_t n;
        int buf = prev.buf ^ 1;
        int e = 0;
        bool hard = false;
        for (;;) {
            const uint64_t lim = ((uint64_t)lb + sh.win) << lp; /* first byte not covered */
            kw = lim >= fsize + GR_LA ? kend : (lim > GR_LA ? (lim - GR_LA) / CH : 0);
            if (kw > kend) kw = kend;
            if (kw <= k) kw = k + 1; /* a window always holds at least one chunk */
            uint64_t endb = kw * CH + GR_LA;
            if (endb > fsize) endb = fsize;
            n = (uint32_t)(((endb + pmask) >> lp) - lb);
            if (n > GR_WIN) { kw = k + 1; endb = kw * CH + GR_LA < fsize ? kw * CH + GR_LA : fsize; n = (uint32_t)(((endb + pmask) >> lp) - lb); }
            e = pin_pages(S, sh, buf, P.fds[f], lb, n, hard ? false : true);
            if (e == -GFS_ENOMEM && !hard) {
                /* the pool is short: shrink the window; at the smallest
                 * window drop the previous one first, then wait for frames */
                if (sh.win > minwin) {
                    if (lane == 0) sh.win = sh.win / 2 > minwin ? sh.win / 2 : minwin;
                } else if (prev.live) {
                    if (lane == 0) wait_phase(sh, P, &sh.full[prev.last_g % GR_STAGES], (prev.last_g / GR_STAGES) & 1u, 7);
                    __syncwarp();
                    unpin_window(S, sh, prev);
                } else {
                    hard = true;
                }
                __syncwarp();
                continue;
            }
            break;
        }
        if (e) {
            if (lane == 0) fail(sh, P, e, 2);
            __syncwarp();
            return false;
        }
        /* the previous window's copies have all landed once its last
         * chunk's full phase completed (its stage is not re-armed yet) */
        if (prev.live) {
            if (lane == 0) wait_phase(sh, P, &sh.full[prev.last_g % GR_STAGES], (prev.last_g / GR_STAGES) & 1u, 3);
            __syncwarp();
            unpin_window(S, sh, prev);
        }
        for (uint64_t kk = k; kk < kw; kk++, g++) {
            const uint32_t s = g % GR_STAGES;
            if (lane == 0) {
                bool ok = true;
                if (g >= GR_STAGES) ok = wait_phase(sh, P, &sh.empty[s], ((g / GR_STAGES) - 1u) & 1u, 4);
                const uint64_t pos = kk * CH;
                const uint64_t rem = fsize - pos;
                StageDesc& dsc = sh.desc[s];
                dsc.pos = pos;
                dsc.f = f;
                dsc.fseq = fseq;
                dsc.clen = (uint32_t)(rem < CH ? rem : CH);
                dsc.avail = (uint32_t)(rem < (uint64_t)CH + GR_LA ? rem : (uint64_t)CH + GR_LA);
                uint8_t* dst = stages + (size_t)s * GR_STAGE;
                if (!ok || sh.abort) {
                    mbar_arrive(&sh.full[s]); /* release the consumers; they see abort */
                } else {
                    const uint32_t body = (dsc.avail + 15u) & ~15u;
                    const uint32_t lbb = pos > 0 ? (uint32_t)GR_LB : 0u;
                    fence_proxy_async();
                    mbar_expect_tx(&sh.full[s], lbb + body);
                    uint64_t from = pos - lbb;
                    uint32_t done = 0, total = lbb + body;
                    while (done < total) {
                        const uint64_t q = from + done;
                        const uint32_t pg = (uint32_t)(q >> lp);
                        const uint32_t inpg = (uint32_t)(q & pmask);
                        uint32_t piece = page - inpg;
                        if (piece > total - done) piece = total - done;
                        const uint8_t* src = S->pool + ((size_t)sh.frames[buf][pg - lb] << lp) + inpg;
                        bulk_g2s(dst + (GR_LB - lbb) + done, src, piece, &sh.full[s]);
                        done += piece;
                    }
                    /* the chunk GR_PF ahead (inside this window) into L2, so
                     * its copy finds it there: the stage ring alone holds
                     * few bytes in flight against HBM latency */
                    if (kk + GR_PF < kw) {
                        const uint64_t pa = (kk + GR_PF) * CH;
                        uint64_t pe = pa + CH < fsize ? pa + CH : fsize;
                        pe = (pe + 15u) & ~15ull;
                        for (uint64_t q = pa; q < pe;) {
                            const uint32_t pg = (uint32_t)(q >> lp);
                            const uint32_t inpg = (uint32_t)(q & pmask);
                            uint32_t piece = page - inpg;
                            if (piece > pe - q) piece = (uint32_t)(pe - q);
                            if (pg - lb < n)
                                bulk_prefetch_l2(S->pool + ((size_t)sh.frames[buf][pg - lb] << lp) + inpg, piece);
                            q += piece;
                        }
                    }
                }
            }
            __syncwarp();
        }
        prev.lb = lb;
        prev.n = n;
        prev.buf = buf;
        prev.last_g = g - 1u;
        prev.live = true;
        k = kw;
        if (sh.abort) return false;
    }
    return true;
}

/* A stage with no bytes (an empty file, or f = -1: the end of a batched
 * CTA's work): published by arriving on its full barrier without a copy. */
__device__ void emit_marker(const GrepDev& P, Shared& sh, int f, uint32_t fseq, uint32_t& g) {
    const int lane = threadIdx.x & 31;
    const uint32_t s = g % GR_STAGES;
    if (lane == 0) {
        if (g >= GR_STAGES) wait_phase(sh, P, &sh.empty[s], ((g / GR_STAGES) - 1u) & 1u, 6);
        StageDesc& dsc = sh.desc[s];
        dsc.pos = 0;
        dsc.f = f;
        dsc.fseq = fseq;
        dsc.clen = 0;
        dsc.avail = 0;
        mbar_arrive(&sh.full[s]);
    }
    __syncwarp();
    g++;
}

/* Producer of the plain scan: the CTA's static run of chunks [c0, c1) of
 * the concatenated corpus. */
__device__ __noinline__ void producer(gfs_state* S, const GrepDev& P, Shared& sh, uint8_t* stages, uint64_t c0, uint64_t c1) {
    const int lane = threadIdx.x & 31;
    Window prev = {0, 0, 1, 0, false};
    uint32_t g = 0;
    uint64_t c = c0;
    while (c < c1) {
        const int f = file_of(P, c);
        const uint64_t kend = (P.chunk_prefix[f + 1] < c1 ? P.chunk_prefix[f + 1] : c1) - P.chunk_prefix[f];
        if (!stream_file<GR_CH>(S, P, sh, stages, f, 0u, c - P.chunk_prefix[f], kend, prev, g)) break;
        c = P.chunk_prefix[f] + kend;
    }
    release_window(S, P, sh, prev, 5);
    /* chunks never produced after an abort: release their consumers */
    if (sh.abort && lane == 0) {
        uint64_t total = c1 - c0;
        for (; g < total; g++) {
            const uint32_t s = g % GR_STAGES;
            if (g >= GR_STAGES && !wait_phase(sh, P, &sh.empty[s], ((g / GR_STAGES) - 1u) & 1u, 6)) {
                /* consumers are gone too */
            }
            mbar_arrive(&sh.full[s]);
        }
    }
}

/* Producer of the batched scan: whole files from the shared queue (longest
 * first), each numbered in sequence for the consumers' per-file flushes;
 * an empty file is one empty stage (the hasher still finishes its XXH64);
 * the end is an f = -1 stage numbered one past the last file. */
__device__ __noinline__ void producer_batch(gfs_state* S, const GrepDev& P, Shared& sh, uint8_t* stages) {
    const int lane = threadIdx.x & 31;
    Window prev = {0, 0, 1, 0, false};
    uint32_t g = 0, fseq = 0;
    for (;;) {
        int f = -1;
        if (lane == 0) {
            const uint32_t i = atomicAdd(P.file_next, 1u);
            f = i < (uint32_t)P.n_files ? P.file_order[i] : -1;
        }
        f = __shfl_sync(0xFFFFFFFFu, f, 0);
        if (f < 0 || sh.abort) break;
        if (lane == 0) sh.fileseq[fseq & 7u] = f;
        __syncwarp();
        const uint64_t nch = (P.sizes[f] + GR_CH_B - 1) / GR_CH_B;
        if (nch == 0) emit_marker(P, sh, f, fseq, g);
        else if (!stream_file<GR_CH_B>(S, P, sh, stages, f, fseq, 0, nch, prev, g)) break;
        fseq++;
    }
    release_window(S, P, sh, prev, 5);
    emit_marker(P, sh, -1, fseq, g);
}

} // namespace

/* The batched scan's consumer barrier (the n-th one a warp passes): an
 * mbarrier of NC arrivals with a bounded wait, so a warp that gave up
 * (timeout, abort) cannot leave the others waiting forever.  false: give up. */
__device__ __forceinline__ bool cbar_wait(Shared& sh, const GrepDev& P, uint32_t n) {
    __syncwarp();
    bool ok = true;
    if ((threadIdx.x & 31) == 0) {
        mbar_arrive(&sh.cbar);
        ok = wait_phase(sh, P, &sh.cbar, n & 1u, 9);
    }
    return __shfl_sync(0xFFFFFFFFu, ok ? 1 : 0, 0) != 0;
}

/* The batched scan's hasher warp: the XXH64 of each file, over the staged
 * chunks in order (chunks are whole 32-byte stripes except a file's last),
 * lanes 0..3 carrying the four accumulators; it releases every stage it has
 * read like a consumer. */
__device__ __noinline__ void hasher(const GrepDev& P, Shared& sh, uint8_t* stages) {
    const int lane = threadIdx.x & 31;
    uint64_t v = gfsx::acc_init(lane & 3);
    for (uint32_t g = 0;; g++) {
        const uint32_t s = g % GR_STAGES;
        bool ok = true;
        if (lane == 0) ok = wait_phase(sh, P, &sh.full[s], (g / GR_STAGES) & 1u, 8);
        ok = __shfl_sync(0xFFFFFFFFu, ok ? 1 : 0, 0) != 0;
        const StageDesc d = sh.desc[s];
        if (!ok || d.f < 0) return;
        if (!sh.abort) {
            const uint8_t* base = stages + (size_t)s * GR_STAGE + GR_LB;
            if (d.pos == 0) v = gfsx::acc_init(lane & 3);
            const uint32_t stripes = d.clen / 32u;
            if (lane < 4) v = gfsx::acc_stripes(v, base, stripes, lane);
            const uint64_t size = P.sizes[d.f];
            if (d.pos + d.clen == size) {
                const uint64_t v1 = __shfl_sync(0xFFFFFFFFu, v, 0), v2 = __shfl_sync(0xFFFFFFFFu, v, 1),
                               v3 = __shfl_sync(0xFFFFFFFFu, v, 2), v4 = __shfl_sync(0xFFFFFFFFu, v, 3);
                if (lane == 0) P.xxh[d.f] = gfsx::finish(v1, v2, v3, v4, size, base + (size_t)stripes * 32u);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&sh.empty[s]);
    }
}

/* Direct scan: each consumer warp loads the window of its own segment --
 * the segment, GR_LB bytes before it and GR_LA + 32 after -- into a private
 * shared buffer and scans it there; no producer, no stage ring.  Bytes come
 * from the file's registered host mapping (16-byte loads over the host
 * link, many warps in flight) or, for a file without one, from its pages
 * in the buffer cache, pinned by lane 0 for the copy.  Bytes outside the
 * file read as zero.  false: failed (the CTA is aborting). */
#define GR_DWIN (GR_LB + GR_SEG + GR_LA + 32) /* bytes per warp window (39 x 16) */
static_assert(GR_DWIN % 16 == 0 && GR_CONS * GR_DWIN <= GR_STAGES * GR_STAGE, "direct windows live in the stage ring");
/* The 16-byte unit at file offset off (a multiple of 16) of a file of fsize
 * bytes, read from q (where that offset's bytes live); zero outside the
 * file. */
__device__ __forceinline__ uint4 window_unit(const uint8_t* q, int64_t off, uint64_t fsize) {
    if (off < 0 || off >= (int64_t)fsize) return make_uint4(0u, 0u, 0u, 0u);
    if (off + 16 <= (int64_t)fsize) return *(const uint4*)q;
    /* the file's last partial unit, byte by byte */
    uint64_t lo = 0, hi = 0;
    const int n = (int)((int64_t)fsize - off);
    for (int i = 0; i < n; i++) {
        const uint64_t b = q[i];
        if (i < 8) lo |= b << (8 * i);
        else hi |= b << (8 * (i - 8));
    }
    return make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
}

/* The window at file position p of a file with a registered host mapping:
 * both of a lane's units are loaded before either is stored (a store to the
 * window could otherwise hold the second load behind the first one's round
 * trip over the host link). */
static_assert(GR_DWIN / 16 <= 64, "two 16-byte units per lane");
__device__ __forceinline__ void load_mapped_window(const GrepDev& P, int f, uint64_t p, uint8_t* buf) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t fsize = P.sizes[f];
    const int64_t first = (int64_t)p - GR_LB;
    const uint8_t* src = (const uint8_t*)P.maps[f];
    const int64_t o0 = first + 16 * (int64_t)lane, o1 = o0 + 16 * 32;
    const uint4 v0 = window_unit(src + o0, o0, fsize);
    const uint4 v1 = lane + 32u < GR_DWIN / 16u ? window_unit(src + o1, o1, fsize) : make_uint4(0u, 0u, 0u, 0u);
    *(uint4*)(buf + 16u * lane) = v0;
    if (lane + 32u < GR_DWIN / 16u) *(uint4*)(buf + 16u * (lane + 32u)) = v1;
}

/* The window of a file without a mapping, from its buffer-cache pages. */
__device__ __noinline__ bool load_window(gfs_state* S, const GrepDev& P, Shared& sh, int f, uint64_t p, uint8_t* buf) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t fsize = P.sizes[f];
    const int64_t first = (int64_t)p - GR_LB; /* file offset of buf[0] */
    const uint8_t* src = (const uint8_t*)P.maps[f];
    uint32_t fr0 = 0, fr1 = 0, pg0 = 0;
    const uint32_t lp = S->log_page;
    if (!src) {
        /* pages covering the window's bytes inside the file: at most two */
        const uint64_t lo = first > 0 ? (uint64_t)first : 0u;
        const uint64_t hi = first + GR_DWIN < (int64_t)fsize ? (uint64_t)(first + GR_DWIN) : fsize;
        int e = 0;
        if (lane == 0 && lo < hi) {
            const PinFile pf = pin_file(S, P.fds[f]);
            bool fresh = false;
            pg0 = (uint32_t)(lo >> lp);
            const uint32_t pg1 = (uint32_t)((hi - 1u) >> lp);
            int r0 = pin_page(S, pf, pg0, GFS_PIN_READ, &fresh);
            int r1 = r0;
            if (r0 >= 0 && pg1 != pg0) {
                r1 = pin_page(S, pf, pg1, GFS_PIN_READ, &fresh);
                if (r1 < 0) unpin(S, (uint32_t)r0);
            }
            e = r0 < 0 ? r0 : (r1 < 0 ? r1 : 0);
            if (e) fail(sh, P, e, 10);
            fr0 = (uint32_t)r0;
            fr1 = (uint32_t)r1;
        }
        e = __shfl_sync(0xFFFFFFFFu, e, 0);
        if (e) return false;
        fr0 = __shfl_sync(0xFFFFFFFFu, fr0, 0);
        fr1 = __shfl_sync(0xFFFFFFFFu, fr1, 0);
        pg0 = __shfl_sync(0xFFFFFFFFu, pg0, 0);
    }
    for (uint32_t u = lane; u < GR_DWIN / 16u; u += 32u) {
        const int64_t off = first + 16 * (int64_t)u;
        /* 16-byte units never straddle a page (pages are >= 4 KiB) */
        const uint8_t* q = src ? src + off
                               : S->pool + ((size_t)((uint32_t)(off >> lp) == pg0 ? fr0 : fr1) << lp) +
                                     ((uint64_t)off & ((1ull << lp) - 1u));
        *(uint4*)(buf + 16u * u) = window_unit(q, off, fsize);
    }
    __syncwarp();
    if (!src && lane == 0 && fsize > 0) {
        const uint64_t lo = first > 0 ? (uint64_t)first : 0u;
        const uint64_t hi = first + GR_DWIN < (int64_t)fsize ? (uint64_t)(first + GR_DWIN) : fsize;
        if (lo < hi) {
            unpin(S, fr0);
            if ((uint32_t)((hi - 1u) >> lp) != pg0) unpin(S, fr1);
        }
    }
    return true;
}

/* Direct scan, warp 31 (no producer there): walks the CTA's chunks up to
 * GR_DPF chunks ahead of the consumers' item counter and asks L2 to fetch
 * each chunk's bytes from the file's host mapping, so the consumers' window
 * loads meet lines already on their way.  Purely a hint: it reads nothing
 * into registers, and gives up quietly on abort or when the consumers stop
 * moving for the session timeout. */
#define GR_DPF 4
__device__ __noinline__ void direct_prefetch(const GrepDev& P, Shared& sh, uint64_t c0, uint64_t c1) {
    const uint32_t lane = threadIdx.x & 31u;
    int f = file_of(P, c0);
    for (uint64_t k = c0; k < c1; k++) {
        Waiter w(sh.wait_ns);
        while (c0 + *(volatile uint32_t*)&sh.next_item / GR_CONS + GR_DPF <= k) {
            if (sh.abort || !w.tick(256)) return;
        }
        while (k >= P.chunk_prefix[f + 1]) f++;
        const uint8_t* src = (const uint8_t*)P.maps[f];
        if (!src) continue;
        const uint64_t pos = (k - P.chunk_prefix[f]) * GR_CH, size = P.sizes[f];
        const uint64_t end = pos + GR_CH + GR_LA < size ? pos + GR_CH + GR_LA : size;
        for (uint64_t o = pos + 128u * lane; o < end; o += 32u * 128u)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(src + o));
    }
}

/* One persistent 1024-thread CTA per SM: warp 31 pins pages and streams
 * chunks (TMA), warps 0..30 scan them; see the file comment.  BATCH: the
 * CTA takes whole files from a shared queue instead of a static run of
 * chunks, warps 0..29 scan and warp 30 computes each file's XXH64. */
template <bool SMEM, bool BATCH, bool DIRECT>
__global__ void __launch_bounds__(GR_THREADS, 1) k_grep_scan(gfs_state* S, GrepDev P) {
    constexpr int NC = BATCH ? GR_CONS_B : GR_CONS;
    constexpr uint32_t CH = (uint32_t)NC * GR_SEG;
    extern __shared__ __align__(128) uint8_t dsm[];
    __shared__ Shared sh;
    /* shared memory: slot tags, displacements, slot counters, the stage
     * ring, per-warp scratch */
    const uint32_t tag_bytes = SMEM ? grep_tag_smem(P.m) : 0u;
    const uint32_t disp_bytes = SMEM ? grep_disp_smem(P.r) : 0u;
    const uint32_t tbl_bytes = SMEM ? tag_bytes + disp_bytes + grep_cnt_smem(P.m) : 0u;
    Tbl tbl;
    tbl.tags = SMEM ? (const uint16_t*)dsm : P.tags;
    tbl.disp = SMEM ? (const uint16_t*)(dsm + tag_bytes) : P.disp;
    tbl.cnt = SMEM ? (uint32_t*)(dsm + tag_bytes + disp_bytes) : nullptr;
    uint8_t* stages = dsm + tbl_bytes;
    uint8_t* wscr = stages + GR_STAGES * GR_STAGE + (size_t)(threadIdx.x >> 5) * GR_WSCR;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if constexpr (SMEM) {
        /* the plan's global tags and displacements are zero padded to these
         * sizes (multiples of 128 bytes) */
        for (uint32_t i = threadIdx.x; i < tag_bytes / 16u; i += blockDim.x)
            ((uint4*)dsm)[i] = __ldg((const uint4*)P.tags + i);
        for (uint32_t i = threadIdx.x; i < disp_bytes / 16u; i += blockDim.x)
            ((uint4*)(dsm + tag_bytes))[i] = __ldg((const uint4*)P.disp + i);
        for (uint32_t i = threadIdx.x; i < grep_cnt_smem(P.m) / 16u; i += blockDim.x)
            ((uint4*)tbl.cnt)[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < GR_STAGES; s++) {
            mbar_init(&sh.full[s], 1u);
            mbar_init(&sh.empty[s], (uint32_t)NC + (BATCH ? 1u : 0u));
        }
        mbar_init(&sh.cbar, (uint32_t)NC);
        fence_mbar_init();
        sh.abort = 0;
        sh.err = 0;
        sh.next_item = 0;
        for (uint32_t L = 0; L <= 16u; L++) {
            uint32_t mw[4];
            for (uint32_t i = 0; i < 4u; i++) {
                const int b = (int)L * 8 - 32 * (int)i;
                mw[i] = b >= 32 ? 0xFFFFFFFFu : (b <= 0 ? 0u : (1u << b) - 1u);
            }
            sh.kmask[L] = make_uint4(mw[0], mw[1], mw[2], mw[3]);
        }
        sh.wait_ns = S->timeout_ns;
        uint32_t w = P.win_pages ? P.win_pages : GR_WIN;
        const uint32_t mw = (uint32_t)((GR_LB + CH + GR_LA + S->page_size - 1) / S->page_size) + 1u;
        sh.win = w > GR_WIN ? GR_WIN : (w < mw ? mw : w);
    }
    __syncthreads();

    if (BATCH) {
        if (warp == 31) { producer_batch(S, P, sh, stages); return; }
        if (warp == NC) { hasher(P, sh, stages); return; }
        /* Items (chunk, segment) in order from the shared counter, as below;
         * file boundaries come from the stages: each file is numbered in
         * sequence, and a warp whose item has a higher number first passes
         * one flush barrier per file in between, so every warp passes the
         * same barriers in the same order even if it saw none of a small
         * file's chunks.  The end marker (f = -1) is numbered one past the
         * last file, which flushes it. */
        uint32_t cur = 0, nbar = 0;
        for (;;) {
            uint32_t it = 0;
            if (lane == 0) it = atomicAdd(&sh.next_item, 1u);
            it = __shfl_sync(0xFFFFFFFFu, it, 0);
            const uint32_t g = it / NC, s = g % GR_STAGES;
            bool ok = true;
            if (lane == 0) ok = wait_phase(sh, P, &sh.full[s], (g / GR_STAGES) & 1u, 1);
            ok = __shfl_sync(0xFFFFFFFFu, ok ? 1 : 0, 0) != 0;
            if (!ok) return; /* gave up: the others see the abort in their waits */
            const StageDesc d = sh.desc[s];
            while (cur < d.fseq) {
                if (!cbar_wait(sh, P, nbar++)) return;
                if (!sh.abort) flush_counts<SMEM, NC>(P, tbl, sh.fileseq[cur & 7u]);
                if (!cbar_wait(sh, P, nbar++)) return;
                cur++;
            }
            if (d.f < 0) return;
            if (!sh.abort) {
                CountSink sink{P, tbl, SMEM, d.f};
                scan_segment<SMEM>(P, tbl, stages + (size_t)s * GR_STAGE + GR_LB, d, it % NC, wscr, sh.kmask, sink);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&sh.empty[s]);
        }
    }

    const uint64_t total = P.total_chunks;
    const uint64_t c0 = total * blockIdx.x / gridDim.x, c1 = total * (blockIdx.x + 1) / gridDim.x;
    if (warp == GR_CONS) {
        if (!DIRECT) producer(S, P, sh, stages, c0, c1);
        else direct_prefetch(P, sh, c0, c1);
        return;
    }
    /* Items (chunk, segment) are taken in order from a shared counter, so a
     * warp that finishes early takes the next segment instead of idling
     * behind the slowest warp of its chunk.  A chunk has exactly NC items,
     * one per consumer warp: a chunk's items cannot all be finished before
     * it has landed, so no warp can take an item of the chunk GR_STAGES
     * stages later while its stage still holds an earlier phase (the parity
     * waits stay unambiguous).  Counts are flushed per file: a warp whose
     * item lies beyond the current file waits at the consumers' barrier,
     * which every warp passes once per file in the same order. */
    const uint32_t nchunks = (uint32_t)(c1 - c0), n_items = nchunks * NC;
    if (nchunks == 0) return;
    int f = file_of(P, c0);
    uint32_t fend = (uint32_t)((P.chunk_prefix[f + 1] < c1 ? P.chunk_prefix[f + 1] : c1) - c0);
    for (;;) {
        uint32_t it = 0;
        if (lane == 0) it = atomicAdd(&sh.next_item, 1u);
        it = __shfl_sync(0xFFFFFFFFu, it, 0);
        const uint32_t g = it < n_items ? it / NC : nchunks;
        while (g >= fend) {
            consumers_sync<NC>();
            if (!sh.abort) flush_counts<SMEM, NC>(P, tbl, f);
            consumers_sync<NC>();
            if (fend >= nchunks) return;
            f = file_of(P, c0 + fend);
            fend = (uint32_t)((P.chunk_prefix[f + 1] < c1 ? P.chunk_prefix[f + 1] : c1) - c0);
        }
        if (DIRECT) {
            /* chunk c0 + g lies in file f (the loop above moved f on) */
            StageDesc d;
            d.f = f;
            d.fseq = 0;
            d.pos = (c0 + g - P.chunk_prefix[f]) * GR_CH;
            const uint64_t rem = P.sizes[f] - d.pos;
            d.clen = (uint32_t)(rem < GR_CH ? rem : GR_CH);
            d.avail = (uint32_t)(rem < (uint64_t)GR_CH + GR_LA ? rem : (uint64_t)GR_CH + GR_LA);
            const uint32_t seg0 = (it % NC) * GR_SEG;
            if (seg0 < d.clen && !sh.abort) {
                uint8_t* buf = stages + (size_t)warp * GR_DWIN;
                bool ok = true;
                if (P.maps[f]) load_mapped_window(P, f, d.pos + seg0, buf);
                else ok = load_window(S, P, sh, f, d.pos + seg0, buf);
                if (ok) {
                    CountSink sink{P, tbl, SMEM, f};
                    scan_segment<SMEM>(P, tbl, buf + GR_LB - seg0, d, it % NC, wscr, sh.kmask, sink);
                }
            }
            __syncwarp();
            continue;
        }
        const uint32_t s = g % GR_STAGES;
        bool ok = true;
        if (lane == 0) ok = wait_phase(sh, P, &sh.full[s], (g / GR_STAGES) & 1u, 1);
        ok = __shfl_sync(0xFFFFFFFFu, ok ? 1 : 0, 0) != 0;
        if (ok && !sh.abort) {
            const StageDesc d = sh.desc[s];
            CountSink sink{P, tbl, SMEM, d.f};
            scan_segment<SMEM>(P, tbl, stages + (size_t)s * GR_STAGE + GR_LB, d, it % NC, wscr, sh.kmask, sink);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&sh.empty[s]);
    }
}

/* ------------------------------------------------------------------ */
/* fix-up: restate the reference chunk walk for files with long runs   */
/* ------------------------------------------------------------------ */
namespace {
struct PageCursor {
    gfs_state* S;
    PinFile pf;
    uint32_t page = 0xFFFFFFFFu;
    int fr = -1;
    __device__ int byte(uint64_t q) {
        if (q >= pf.size) return 0;
        uint32_t pg = (uint32_t)(q >> S->log_page);
        if (pg != page) {
            if (fr >= 0) unpin(S, (uint32_t)fr);
            bool fresh;
            fr = pin_page(S, pf, pg, GFS_PIN_READ, &fresh);
            if (fr >= 0 && fresh) publish_valid(S, (uint32_t)fr);
            page = fr >= 0 ? pg : 0xFFFFFFFFu;
            if (fr < 0) return -1;
        }
        return (int)__ldcg(S->pool + ((size_t)fr << S->log_page) + (q & (S->page_size - 1u)));
    }
    __device__ void release() {
        if (fr >= 0) unpin(S, (uint32_t)fr);
        fr = -1;
        page = 0xFFFFFFFFu;
    }
};

__device__ void count_piece(const GrepDev& P, PageCursor& pc, uint64_t a, uint64_t b, int f) {
    int len = (int)(b - a);
    if (len <= 0 || len > 32) return;
    uint8_t buf[40];
    for (int i = 0; i < 40; i++) buf[i] = 0;
    for (int i = 0; i < len; i++) buf[i] = (uint8_t)pc.byte(a + (uint64_t)i);
    uint32_t k[8];
    for (int i = 0; i < 8; i++)
        k[i] = (uint32_t)buf[4 * i] | ((uint32_t)buf[4 * i + 1] << 8) | ((uint32_t)buf[4 * i + 2] << 16) |
               ((uint32_t)buf[4 * i + 3] << 24);
    Tbl t;
    t.tags = P.tags;
    t.disp = P.disp;
    t.cnt = nullptr;
    CountSink sink{P, t, false, f};
    lookup_hit<false>(P, t, k, (uint32_t)len, sink);
}
} // namespace

/* One block per flagged file; thread 0 restates the reference's window walk
 * (16384 + 32 bytes with overlap stitching, grep_text_gpu.cu:298-318).  A
 * window whose 32-byte halo is all letters cuts the alpha run at its end q;
 * the runs so cut (>= 33 letters, counted as nothing by the scan) are split
 * at every such q and the pieces are counted. */
__global__ void k_grep_fixup(gfs_state* S, GrepDev P) {
    const int f = blockIdx.x;
    if (threadIdx.x != 0 || f >= P.n_files || !P.long_flags[f]) return;
    PageCursor pc;
    pc.S = S;
    pc.pf = pin_file(S, P.fds[f]);
    const uint64_t size = P.sizes[f];
    uint64_t cursor = 0, rs = 0, re = 0, a = 0;
    bool have_run = false;
    while (cursor < size && size - cursor >= 16416ull) {
        int overlap = 0;
        while (overlap < 32) {
            int c = pc.byte(cursor + 16384ull + (uint64_t)overlap);
            if (c < 0) { atomicOr(P.status, GFS_ERRB_IO); pc.release(); return; }
            if (!is_alpha((uint32_t)c)) break;
            overlap++;
        }
        if (overlap == 32) {
            const uint64_t q = cursor + 16416ull;
            if (q < size && is_alpha((uint32_t)pc.byte(q))) {
                if (!have_run || q >= re) {
                    if (have_run) count_piece(P, pc, a, re, f);
                    rs = q - 32ull;
                    while (rs > 0 && is_alpha((uint32_t)pc.byte(rs - 1))) rs--;
                    re = q;
                    while (re < size && is_alpha((uint32_t)pc.byte(re))) re++;
                    a = rs;
                    have_run = true;
                }
                count_piece(P, pc, a, q, f);
                a = q;
            }
        }
        cursor += 16384ull + (uint64_t)overlap;
    }
    if (have_run) count_piece(P, pc, a, re, f);
    pc.release();
}

/* One block per file; thread 0 counts the tokens of [tail_start, size) once
 * more.  The reference's walk moves its cursor by 16384 after its last
 * window too (grep_text_gpu.cu:318), so when that window is longer than
 * 16384 bytes the loop goes round again and reads the bytes past the cursor
 * (at most 31) as a window of their own: their alpha runs, cut at the
 * window's start, are counted a second time.  The host finds tail_start by
 * the same walk. */
static __global__ void k_grep_tail(gfs_state* S, GrepDev P) {
    const int f = blockIdx.x;
    if (threadIdx.x != 0 || f >= P.n_files) return;
    const uint64_t size = P.sizes[f];
    uint64_t q = P.tail_start[f];
    if (q >= size) return;
    PageCursor pc;
    pc.S = S;
    pc.pf = pin_file(S, P.fds[f]);
    while (q < size) {
        const int c = pc.byte(q);
        if (c < 0) {
            atomicOr(P.status, GFS_ERRB_IO);
            break;
        }
        if (!is_alpha((uint32_t)c)) {
            q++;
            continue;
        }
        uint64_t e = q + 1u;
        int ce = 0;
        while (e < size && (ce = pc.byte(e)) >= 0 && is_alpha((uint32_t)ce)) e++;
        if (ce < 0) {
            atomicOr(P.status, GFS_ERRB_IO);
            break;
        }
        count_piece(P, pc, q, e, f);
        q = e;
    }
    pc.release();
}

template __global__ void k_grep_scan<true, false, false>(gfs_state*, GrepDev);
template __global__ void k_grep_scan<false, false, false>(gfs_state*, GrepDev);
template __global__ void k_grep_scan<true, true, false>(gfs_state*, GrepDev);
template __global__ void k_grep_scan<false, true, false>(gfs_state*, GrepDev);
template __global__ void k_grep_scan<true, false, true>(gfs_state*, GrepDev);
template __global__ void k_grep_scan<false, false, true>(gfs_state*, GrepDev);

/* ------------------------------------------------------------------ */
/* host side: dictionary table, file opening, launch                   */
/* ------------------------------------------------------------------ */
/* ------------------------------------------------------------------ */
/* served loop: a persistent kernel whose warps take requests from a    */
/* ring in mapped host memory and serve them through the buffer cache  */
/* ------------------------------------------------------------------ */
struct SvReq { /* ring slot: the host fills it, then publishes seq = ticket + 1 */
    uint32_t seq;
    uint32_t op;
    uint32_t file;
    uint32_t id;
    uint64_t offset;
    uint64_t length;
};
struct SvComp { /* completion, indexed by request id: done is written last */
    unsigned long long result;
    int status;
    uint32_t done;
};
/* A large grep request is split into parts that any serving warp may take
 * (a part is a run of the request's 512-byte segments); the request's
 * accumulator collects the parts' counts and the part that finishes last
 * publishes the completion. */
struct SvAcc {
    unsigned long long count;
    uint32_t left;         /* parts not finished */
    int status;            /* the first part's error */
    unsigned long long t0; /* %globaltimer when a warp took the request */
};
#define SV_HIST 64 /* service-time histogram: bucket b counts times in [2^b, 2^(b+1)) ns */
struct SvPart { /* a slot of the part queue (sequence protocol as the ring) */
    uint32_t seq;
    uint32_t id, file, unused;
    uint64_t off, end;       /* the request's range */
    uint64_t seg_lo, seg_hi; /* this part's segments: [seg_lo, seg_hi) in steps of 512 */
};
#define SV_QCAP 16384u          /* part queue slots (power of two) */
#define SV_SPLIT (1ull << 20)   /* greps longer than this are split ... */
#define SV_PART (256ull << 10)  /* ... into parts of about this many bytes ... */
#define SV_MAXP 64u             /* ... and at most this many */
struct ServeDev {
    GrepDev G;              /* the dictionary (table in global memory) */
    SvReq* ring;            /* device view of the mapped ring */
    uint32_t ring_mask;
    uint32_t* head;         /* next ticket (device memory) */
    SvComp* comp;           /* device view of the mapped completions */
    const int* fds;         /* served files, opened once for the server's life */
    const uint64_t* sizes;
    const int* out_fds;     /* output files (write-once) */
    int n_files, n_out;
    const uint32_t* stop;   /* mapped: set by the host when every request is done */
    SvAcc* acc;             /* per request id (device memory, zeroed per run) */
    SvPart* parts;          /* SV_QCAP slots */
    uint32_t* q_head;       /* next part to take */
    uint32_t* q_tail;       /* next part position to reserve */
    uint32_t tbl_smem;      /* bytes of slot tags + displacements staged in each block's
                               dynamic shared memory (0: read from global memory) */
    unsigned long long* hist; /* SV_HIST buckets of device service time (device memory) */
};
#define SV_WARPS 8
#define SV_STAGE (GR_LB + GR_SEG + GR_LA + 16)

namespace {

__device__ __forceinline__ uint32_t sv_pattern(uint64_t x, uint32_t id) {
    /* byte x of a served write: a fixed function of the file offset and request */
    return (uint32_t)(((uint32_t)x * 0x9E3779B1u + id * 0x85EBCA77u) >> 24);
}

/* A warp's window of up to `batch` pinned pages of one file, lane j holding
 * page lo + j, so the misses of a large request are in flight together; a
 * pool short of frames makes it fall back to windows of at most two pages
 * whose pins wait for frames.  cover() slides it to start at page pa so
 * that it holds pages pa..pb (pb <= pa + 1, the pages of one piece). */
struct PageWindow {
    PinFile pf;
    uint32_t lo = 0, nw = 0, batch = 8, last = 0;
    int fr = -1;
    __device__ int cover(gfs_state* S, uint32_t pa, uint32_t pb) {
        if (nw != 0 && pa >= lo && pb < lo + nw) return 0;
        const uint32_t lane = threadIdx.x & 31u;
        for (;;) {
            if (lane < nw) unpin(S, (uint32_t)fr);
            nw = last - pa + 1u < batch ? last - pa + 1u : batch;
            if (nw < pb - pa + 1u) nw = pb - pa + 1u;
            lo = pa;
            fr = -1;
            if (lane < nw) {
                bool fresh;
                fr = pin_page(S, pf, lo + lane, GFS_PIN_READ | (nw > 2 ? GFS_PIN_NOALLOC : 0), &fresh);
                if (fr >= 0 && fresh) publish_valid(S, (uint32_t)fr);
            }
            const unsigned nomem = __ballot_sync(0xFFFFFFFFu, lane < nw && fr == -GFS_ENOMEM);
            const unsigned bad = __ballot_sync(0xFFFFFFFFu, lane < nw && fr < 0 && fr != -GFS_ENOMEM);
            if (!bad && !nomem) return 0;
            if (lane < nw && fr >= 0) unpin(S, (uint32_t)fr);
            nw = 0;
            if (bad) return __shfl_sync(0xFFFFFFFFu, fr, __ffs(bad) - 1);
            if (batch <= 2) return -GFS_ENOMEM;
            batch = 2;
        }
    }
    /* the frame of a page inside the window (every lane calls) */
    __device__ int frame(uint32_t pg) const { return __shfl_sync(0xFFFFFFFFu, fr, (int)(pg - lo)); }
    __device__ void release(gfs_state* S) {
        if ((threadIdx.x & 31u) < nw) unpin(S, (uint32_t)fr);
        nw = 0;
    }
};

/* read + XXH64 of [off, end) of a served file, by one warp, at any offset.
 * Pages are pinned in windows of up to 8 (lane j holds page lo + j), so the
 * misses of a large request are in flight together; a pool short of frames
 * falls back to windows of one page (multi-page pins do not wait for
 * frames).  The range is hashed in logical 512-byte chunks from `off` (so
 * every full chunk is 16 whole stripes): a chunk's bytes are loaded as the
 * 16-byte aligned units of the file that cover it (each inside one page)
 * into `raw`, then shifted into `st` by the chunk's offset within its first
 * unit (funnel shifts of 32-bit words), where lanes 0..3 run the four
 * accumulator lanes over them. */
__device__ int sv_read_xxh(gfs_state* S, const ServeDev& D, int fd, uint64_t off, uint64_t end, uint8_t* st,
                           uint8_t* raw, unsigned long long* result) {
    const int lane = threadIdx.x & 31;
    const uint32_t lp = S->log_page, pmask = S->page_size - 1u;
    PageWindow win;
    win.pf = pin_file(S, fd);
    win.last = end > off ? (uint32_t)((end - 1) >> lp) : 0u;
    uint64_t v = gfsx::acc_init(lane & 3);
    int err = 0;
    const uint8_t* tail = st;
    for (uint64_t pos = off; pos < end;) {
        const uint32_t clen = end - pos < 512u ? (uint32_t)(end - pos) : 512u;
        const uint64_t a0 = pos & ~15ull, cend = pos + clen;
        err = win.cover(S, (uint32_t)(a0 >> lp), (uint32_t)((cend - 1) >> lp));
        if (err) break;
        const uint32_t sh = (uint32_t)(pos & 15u);
        if (sh == 0u) {
            /* an aligned range (every chunk of it is): units straight into st */
            const uint64_t q = a0 + 16ull * (uint32_t)lane;
            const int f = win.frame(q < cend ? (uint32_t)(q >> lp) : win.lo);
            if (q < cend) *(uint4*)(st + 16u * (uint32_t)lane) = ld_cg4(S->pool + ((size_t)f << lp) + (q & pmask));
            __syncwarp();
        } else {
            /* the aligned units covering [pos, cend): at most 33 */
            for (uint32_t u0 = 0; a0 + 16ull * u0 < cend; u0 += 32u) {
                const uint64_t q = a0 + 16ull * (u0 + (uint32_t)lane);
                const int f = win.frame(q < cend ? (uint32_t)(q >> lp) : win.lo);
                if (q < cend)
                    *(uint4*)(raw + 16u * (u0 + (uint32_t)lane)) = ld_cg4(S->pool + ((size_t)f << lp) + (q & pmask));
            }
            __syncwarp();
        }
        /* shift by pos & 15 into st (16 bytes a lane, 512 at most) */
        if (sh != 0u && 16u * (uint32_t)lane < clen) {
            const uint32_t* w = (const uint32_t*)(raw + (sh & ~3u) + 16u * (uint32_t)lane);
            const uint32_t b = 8u * (sh & 3u);
            const uint32_t x0 = w[0], x1 = w[1], x2 = w[2], x3 = w[3], x4 = w[4];
            *(uint4*)(st + 16u * (uint32_t)lane) = make_uint4(__funnelshift_r(x0, x1, b), __funnelshift_r(x1, x2, b),
                                                              __funnelshift_r(x2, x3, b), __funnelshift_r(x3, x4, b));
        }
        __syncwarp();
        const uint32_t stripes = clen / 32u;
        if (lane < 4) v = gfsx::acc_stripes(v, st, stripes, lane);
        tail = st + stripes * 32u;
        pos = cend;
        if (pos < end) __syncwarp();
    }
    win.release(S);
    if (err) return err;
    const uint64_t v1 = __shfl_sync(0xFFFFFFFFu, v, 0), v2 = __shfl_sync(0xFFFFFFFFu, v, 1),
                   v3 = __shfl_sync(0xFFFFFFFFu, v, 2), v4 = __shfl_sync(0xFFFFFFFFu, v, 3);
    if (lane == 0) *result = gfsx::finish(v1, v2, v3, v4, end - off, tail);
    __syncwarp();
    return 0;
}

/* dictionary words among the tokens of [off, end), the range read as a
 * text of its own (bytes outside it are not letters), by one warp */
__device__ int sv_grep(gfs_state* S, const ServeDev& D, int fd, uint64_t off, uint64_t end, uint64_t seg_lo,
                       uint64_t seg_hi, uint8_t* st, uint8_t* wscr, const uint4* km, unsigned long long* result) {
    const int lane = threadIdx.x & 31;
    const uint32_t lp = S->log_page, pmask = S->page_size - 1u;
    PageWindow win;
    win.pf = pin_file(S, fd);
    win.last = seg_hi > seg_lo ? (uint32_t)(((seg_hi + GR_SEG + GR_LA < end ? seg_hi + GR_SEG + GR_LA : end) - 1) >> lp)
                               : 0u;
    /* the table's tags and displacements from the block's shared copy when
     * there is one (generic loads serve either place) */
    extern __shared__ __align__(128) uint8_t sv_dsm[];
    Tbl t;
    t.tags = D.tbl_smem ? (const uint16_t*)sv_dsm : D.G.tags;
    t.disp = D.tbl_smem ? (const uint16_t*)(sv_dsm + grep_tag_smem(D.G.m)) : D.G.disp;
    t.cnt = nullptr;
    TotalSink sink;
    int err = 0;
    /* segments start 16-byte aligned in the file (the staged units are then
     * aligned), at off & ~15 plus multiples of 512; this call scans those in
     * [seg_lo, seg_hi).  Bytes before off or from end on are staged as
     * zeros, which are not letters, so the range reads as a text of its own
     * and a token is counted by the segment it starts in, whichever part
     * that segment falls in. */
    for (uint64_t seg = seg_lo; seg < seg_hi && seg < end; seg += GR_SEG) {
        /* stage [seg - 16, seg + 512 + 64) with bytes outside [off, end) zero */
        const uint64_t lo = seg >= off + GR_LB ? seg - GR_LB : off;
        const uint64_t hi = seg + GR_SEG + GR_LA < end ? seg + GR_SEG + GR_LA : end;
        const int r = win.cover(S, (uint32_t)(lo >> lp), (uint32_t)((hi - 1) >> lp));
        if (r < 0) { err = r; break; }
        for (uint32_t u0 = 0; u0 < (GR_LB + GR_SEG + GR_LA) / 16u; u0 += 32u) {
            const uint32_t u = u0 + (uint32_t)lane;
            const int64_t a = (int64_t)seg - GR_LB + 16 * (int64_t)u; /* file offset of this 16-byte unit */
            const bool in = u < (GR_LB + GR_SEG + GR_LA) / 16u && a + 16 > (int64_t)off && (uint64_t)a < end;
            const int fr = win.frame(in ? (uint32_t)((uint64_t)a >> lp) : win.lo);
            if (u >= (GR_LB + GR_SEG + GR_LA) / 16u) continue;
            uint4 w = make_uint4(0, 0, 0, 0);
            if (in) {
                w = ld_cg4(S->pool + ((size_t)fr << lp) + ((uint64_t)a & pmask));
                const uint64_t rem = end - (uint64_t)a;
                const int64_t skip = (int64_t)off - a; /* bytes before off in this unit */
                if (rem < 16 || skip > 0) { /* zero the bytes outside [off, end) */
                    uint32_t* ww = (uint32_t*)&w;
                    for (int q = 0; q < 4; q++) {
                        const int keep = (int)(rem < 16 ? rem : 16) - 4 * q;
                        uint32_t m = keep >= 4 ? 0xFFFFFFFFu : (keep <= 0 ? 0u : (1u << (8 * keep)) - 1u);
                        const int drop = (int)skip - 4 * q;
                        m &= drop >= 4 ? 0u : (drop <= 0 ? 0xFFFFFFFFu : ~((1u << (8 * drop)) - 1u));
                        ww[q] &= m;
                    }
                }
            }
            *(uint4*)(st + 16 * u) = w;
        }
        __syncwarp();
        StageDesc d;
        d.pos = seg == off ? 0 : 1; /* only its being zero matters: no byte before the range */
        d.f = 0;
        d.fseq = 0;
        d.clen = end - seg < GR_SEG ? (uint32_t)(end - seg) : (uint32_t)GR_SEG;
        d.avail = end - seg < GR_SEG + GR_LA ? (uint32_t)(end - seg) : (uint32_t)(GR_SEG + GR_LA);
        scan_segment<true>(D.G, t, st + GR_LB, d, 0u, wscr, km, sink);
        __syncwarp();
    }
    win.release(S);
    if (err) return err;
    uint32_t n = sink.n;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xFFFFFFFFu, n, o);
    if (lane == 0) *result = n;
    __syncwarp();
    return 0;
}

/* write the request's pattern over [off, off+len) of a write-once output
 * file, page by page (the page-level steps of gwrite), by one warp */
__device__ int sv_write(gfs_state* S, int fd, uint64_t off, uint64_t len, uint32_t id, unsigned long long* result) {
    const int lane = threadIdx.x & 31;
    const uint32_t lp = S->log_page;
    const uint64_t page = 1ull << lp, end = off + len;
    PinFile pf;
    if (lane == 0) pf = pin_file(S, fd);
    for (uint64_t pos = off; pos < end;) {
        const uint64_t pst = pos & ~(page - 1ull), pe = pst + page < end ? pst + page : end;
        int fr = 0;
        bool fresh = false;
        if (lane == 0) {
            const bool full = pos == pst && pe == pst + page;
            fr = pin_page(S, pf, (uint32_t)(pos >> lp), full ? GFS_PIN_WFULL : GFS_PIN_WONCE, &fresh);
        }
        fr = __shfl_sync(0xFFFFFFFFu, fr, 0);
        fresh = __shfl_sync(0xFFFFFFFFu, fresh ? 1 : 0, 0) != 0;
        if (fr < 0) return fr;
        uint8_t* d = frame_data(S, (uint32_t)fr);
        if (fresh) { /* bytes of the page this write does not cover start at zero */
            if (pos > pst) warp_zero(d, pos - pst, lane);
            if (pe < pst + page) warp_zero(d + (pe - pst), pst + page - pe, lane);
        }
        for (uint64_t x = pos + (uint64_t)lane * 4u; x < pe; x += 128u) {
            uint32_t w = 0;
            for (int b = 0; b < 4; b++)
                if (x + (uint64_t)b < pe) w |= (sv_pattern(x + (uint64_t)b, id) & 0xFFu) << (8 * b);
            if (x + 4 <= pe) *(uint32_t*)(d + (x - pst)) = w;
            else for (int b = 0; x + (uint64_t)b < pe; b++) d[x - pst + (uint64_t)b] = (uint8_t)(w >> (8 * b));
        }
        __syncwarp();
        if (lane == 0) {
            __threadfence();
            atomicMax(&S->frames[fr].content, (uint32_t)(pe - pst));
            if (fresh) publish_valid(S, (uint32_t)fr);
            mark_dirty(S, (uint32_t)fr);
            unpin(S, (uint32_t)fr);
            atomicMax((unsigned long long*)&S->files[pf.slot].size, (unsigned long long)pe);
        }
        __syncwarp();
        pos = pe;
    }
    if (lane == 0) *result = len;
    return 0;
}

/* publish a request's completion (lane 0) */
/* publish a request's completion (lane 0), after counting its device
 * service time -- from the take of its ticket's request to now -- in the
 * run's histogram */
__device__ __forceinline__ void sv_complete(const ServeDev& D, uint32_t id, unsigned long long res, int status) {
    const unsigned long long dt = gtimer() - D.acc[id].t0;
    atomicAdd(&D.hist[63 - __clzll((long long)(dt | 1ull))], 1ull);
    SvComp* c = &D.comp[id];
    asm volatile("st.relaxed.sys.global.u64 [%0], %1;" ::"l"(&c->result), "l"(res) : "memory");
    asm volatile("st.relaxed.sys.global.u32 [%0], %1;" ::"l"(&c->status), "r"((uint32_t)status) : "memory");
    st_rel_sys(&c->done, 1u);
}

/* lane 0: one part of a split request is done; the part that finishes last
 * publishes the request's completion with the summed count */
__device__ void sv_part_done(const ServeDev& D, uint32_t id, unsigned long long n, int status) {
    SvAcc* a = &D.acc[id];
    if (status) atomicCAS(&a->status, 0, status);
    atomicAdd(&a->count, n);
    __threadfence();
    if (atomicSub(&a->left, 1u) == 1u) {
        __threadfence();
        const unsigned long long total = atomicAdd(&a->count, 0ull);
        const int st = atomicAdd(&a->status, 0);
        sv_complete(D, id, st ? 0ull : total, st);
    }
}

/* lane 0: take a queued part if there is one (true: *pt holds it) */
__device__ bool sv_take_part(const ServeDev& D, const gfs_state* S, SvPart* pt) {
    for (;;) {
        const uint32_t h = ld_rlx(D.q_head);
        if ((int32_t)(ld_rlx(D.q_tail) - h) <= 0) return false;
        if (atomicCAS(D.q_head, h, h + 1u) != h) continue;
        SvPart* q = &D.parts[h & (SV_QCAP - 1u)];
        /* the producer reserved the position before writing it: wait the
         * few instructions until it is there (bounded all the same) */
        Waiter w(S->timeout_ns);
        while (ld_acq(&q->seq) != h + 1u)
            if (!w.tick(256)) return false;
        *pt = *q;
        __threadfence();
        st_rel(&q->seq, h + SV_QCAP);
        return true;
    }
}

/* lane 0: reserve n consecutive part positions if the queue has room for
 * them (else false: the request is served whole) */
__device__ bool sv_reserve_parts(const ServeDev& D, uint32_t n, uint32_t* pos) {
    for (;;) {
        const uint32_t t = ld_rlx(D.q_tail);
        if (t + n - ld_rlx(D.q_head) > SV_QCAP) return false;
        if (atomicCAS(D.q_tail, t, t + n) == t) {
            *pos = t;
            return true;
        }
    }
}

/* One queued part of a split grep (the whole warp; pt valid in lane 0). */
__device__ __noinline__ void sv_serve_part(gfs_state* S, const ServeDev& D, const SvPart& pt, uint8_t* st,
                                           uint8_t* wscr, const uint4* kmask) {
    const int lane = threadIdx.x & 31;
    const uint32_t id = __shfl_sync(0xFFFFFFFFu, pt.id, 0), file = __shfl_sync(0xFFFFFFFFu, pt.file, 0);
    const uint64_t o = __shfl_sync(0xFFFFFFFFu, pt.off, 0), e = __shfl_sync(0xFFFFFFFFu, pt.end, 0);
    const uint64_t lo = __shfl_sync(0xFFFFFFFFu, pt.seg_lo, 0), hi = __shfl_sync(0xFFFFFFFFu, pt.seg_hi, 0);
    unsigned long long n = 0;
    const int stt = sv_grep(S, D, D.fds[file], o, e, lo, hi, st, wscr, kmask, &n);
    if (lane == 0) sv_part_done(D, id, n, stt);
    __syncwarp();
}

/* A grep request (the whole warp): served whole, or -- longer than SV_SPLIT
 * -- split into parts, all but the first queued for any warp to take.
 * Returns true when split (the completion then comes from the part that
 * finishes last); false with *res and *status set otherwise. */
__device__ __noinline__ bool sv_grep_request(gfs_state* S, const ServeDev& D, uint32_t file, uint32_t id, uint64_t o,
                                             uint64_t e, uint8_t* st, uint8_t* wscr, const uint4* kmask,
                                             unsigned long long* res, int* status) {
    const int lane = threadIdx.x & 31;
    bool split = false;
    const uint64_t s0 = o & ~15ull, nseg = (e - s0 + GR_SEG - 1) / GR_SEG;
    uint32_t np = 1;
    if (e - o > SV_SPLIT) {
        const uint64_t want = (e - o + SV_PART - 1) / SV_PART;
        np = (uint32_t)(want < SV_MAXP ? want : SV_MAXP);
    }
    uint32_t pos = 0;
    if (np > 1) {
        /* the accumulator first, then the queued parts 1..np-1 */
        bool ok = false;
        if (lane == 0) {
            atomicExch(&D.acc[id].count, 0ull);
            atomicExch(&D.acc[id].status, 0);
            atomicExch(&D.acc[id].left, np);
            __threadfence();
            ok = sv_reserve_parts(D, np - 1u, &pos);
        }
        ok = __shfl_sync(0xFFFFFFFFu, ok ? 1 : 0, 0) != 0;
        pos = __shfl_sync(0xFFFFFFFFu, pos, 0);
        if (!ok) np = 1;
    }
    if (np > 1) {
        split = true;
        for (uint32_t k = 1u + (uint32_t)lane; k < np; k += 32u) {
            SvPart* q = &D.parts[(pos + k - 1u) & (SV_QCAP - 1u)];
            /* the slot is free once its last taker has copied it out (it
             * took the position before the reservation, which left room
             * for these): a few instructions */
            Waiter w(S->timeout_ns);
            bool freed = true;
            while (ld_acq(&q->seq) != pos + k - 1u)
                if (!w.tick(256)) { freed = false; break; }
            if (!freed) {
                /* never seen: the part is counted as failed */
                sv_part_done(D, id, 0ull, -GFS_ETIMEDOUT);
                continue;
            }
            q->id = id;
            q->file = file;
            q->off = o;
            q->end = e;
            q->seg_lo = s0 + GR_SEG * (nseg * k / np);
            q->seg_hi = s0 + GR_SEG * (nseg * (k + 1u) / np);
            __threadfence();
            st_rel(&q->seq, pos + k);
        }
        __syncwarp();
        unsigned long long n0 = 0;
        const int st0 = sv_grep(S, D, D.fds[file], o, e, s0, s0 + GR_SEG * (nseg / np), st, wscr, kmask, &n0);
        if (lane == 0) sv_part_done(D, id, n0, st0);
        __syncwarp();
    } else {
        *status = sv_grep(S, D, D.fds[file], o, e, s0, e, st, wscr, kmask, res);
    }
    return split;
}

} // namespace

/* Served loop: each warp takes the next ticket, waits (bounded by the
 * session timeout, or until the host sets stop) for that request, frees
 * its ring slot, serves it and publishes the completion.  A grep longer
 * than SV_SPLIT is split: its warp queues all but the first part, serves
 * the first, and the rest are taken by warps between requests (a warp
 * waiting for its next request serves queued parts meanwhile). */
__global__ void __launch_bounds__(SV_WARPS * 32) k_serve(gfs_state* S, ServeDev D) {
    __shared__ __align__(16) uint8_t stage[SV_WARPS][SV_STAGE];
    __shared__ __align__(16) uint8_t rawb[SV_WARPS][33 * 16 + 16]; /* read requests' aligned units */
    __shared__ __align__(16) uint8_t wscr[SV_WARPS][GR_WSCR];
    __shared__ uint4 kmask[17];
    extern __shared__ __align__(128) uint8_t sv_dsm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x <= 16u) {
        uint32_t mw[4];
        for (uint32_t i = 0; i < 4u; i++) {
            const int b = (int)threadIdx.x * 8 - 32 * (int)i;
            mw[i] = b >= 32 ? 0xFFFFFFFFu : (b <= 0 ? 0u : (1u << b) - 1u);
        }
        kmask[threadIdx.x] = make_uint4(mw[0], mw[1], mw[2], mw[3]);
    }
    /* the dictionary's slot tags and displacements into shared memory (the
     * plan's global copies are zero padded to these sizes): the grep path's
     * two table loads per token then cost a shared-memory access */
    if (D.tbl_smem) {
        const uint32_t tb = grep_tag_smem(D.G.m), db = grep_disp_smem(D.G.r);
        for (uint32_t i = threadIdx.x; i < tb / 16u; i += blockDim.x)
            ((uint4*)sv_dsm)[i] = __ldg((const uint4*)D.G.tags + i);
        for (uint32_t i = threadIdx.x; i < db / 16u; i += blockDim.x)
            ((uint4*)(sv_dsm + tb))[i] = __ldg((const uint4*)D.G.disp + i);
    }
    __syncthreads();
    for (;;) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(D.head, 1u);
        t = __shfl_sync(0xFFFFFFFFu, t, 0);
        SvReq* slot = &D.ring[t & D.ring_mask];
        uint32_t have = 0;
        uint4 a = make_uint4(0, 0, 0, 0), b = make_uint4(0, 0, 0, 0);
        for (;;) {
            /* lane 0 waits for the ticket's request; a queued part found
             * meanwhile is served by the warp (have = 2), then the wait
             * goes on (the idle limit counts from the last work done) */
            SvPart pt;
            if (lane == 0) {
                have = 0;
                const uint64_t t0 = gtimer();
                uint32_t ns = 64, k = 0;
                for (;;) {
                    if (ld_acq_sys(&slot->seq) == t + 1u) { have = 1; break; }
                    if (sv_take_part(D, S, &pt)) { have = 2; break; }
                    if (ld_rlx_sys(D.stop)) break;
                    if ((++k & 63u) == 0u && gtimer() - t0 > S->timeout_ns) break; /* idle too long: leave */
                    __nanosleep(ns);
                    if (ns < 2048) ns <<= 1;
                }
                if (have == 1) {
                    asm volatile("ld.relaxed.sys.global.v4.u32 {%0,%1,%2,%3}, [%4];"
                                 : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w) : "l"(slot) : "memory");
                    asm volatile("ld.relaxed.sys.global.v4.u32 {%0,%1,%2,%3}, [%4];"
                                 : "=r"(b.x), "=r"(b.y), "=r"(b.z), "=r"(b.w) : "l"((const uint8_t*)slot + 16) : "memory");
                    st_rel_sys(&slot->seq, t + D.ring_mask + 1u); /* the slot is free for the host again */
                }
            }
            have = __shfl_sync(0xFFFFFFFFu, have, 0);
            if (have != 2) break;
            sv_serve_part(S, D, pt, stage[warp], wscr[warp], kmask);
        }
        if (!have) return;
        const uint32_t op = __shfl_sync(0xFFFFFFFFu, a.y, 0), file = __shfl_sync(0xFFFFFFFFu, a.z, 0),
                       id = __shfl_sync(0xFFFFFFFFu, a.w, 0);
        if (lane == 0) D.acc[id].t0 = gtimer(); /* ordered before any part of it is queued */
        const uint64_t off = ((uint64_t)__shfl_sync(0xFFFFFFFFu, b.y, 0) << 32) | __shfl_sync(0xFFFFFFFFu, b.x, 0);
        const uint64_t len = ((uint64_t)__shfl_sync(0xFFFFFFFFu, b.w, 0) << 32) | __shfl_sync(0xFFFFFFFFu, b.z, 0);
        unsigned long long res = 0;
        int status = 0;
        bool split = false;
        if (op == GFS_SV_WRITE && (off & 15u)) {
            status = -GFS_EINVAL; /* written ranges start 16-byte aligned (vector stores) */
        } else if (op == GFS_SV_WRITE) {
            status = (int)file < D.n_out ? sv_write(S, D.out_fds[file], off, len, id, &res) : -GFS_EINVAL;
        } else if ((int)file < D.n_files && (op == GFS_SV_READ || op == GFS_SV_GREP)) {
            const uint64_t size = D.sizes[file];
            const uint64_t o = off < size ? off : size, e = len < size - o ? o + len : size;
            if (op == GFS_SV_READ) {
                status = sv_read_xxh(S, D, D.fds[file], o, e, stage[warp], rawb[warp], &res);
            } else {
                split = sv_grep_request(S, D, file, id, o, e, stage[warp], wscr[warp], kmask, &res, &status);
            }
        } else {
            status = -GFS_EINVAL;
        }
        if (lane == 0 && !split) sv_complete(D, id, res, status);
        __syncwarp();
    }
}

/* ---------------- dictionary table built on the device ----------------
 * The same table as the host build (same hashes, tags, geometry), made by
 * five kernels: keys, dedupe, duplicate chains, the seeded displacement
 * search (one cooperative launch), and the table image.  Where several
 * valid displacements exist the device may pick another one than the host;
 * the counts a scan produces do not depend on it. */
struct TbDev {
    const uint8_t* dict; /* n records of 32 bytes */
    int n;
    uint4* klo;          /* key bytes 0..15 / 16..31 per record */
    uint4* khi;
    uint32_t* h1;        /* per record: hash under the current seed */
    int* len;
    int* set;            /* dedupe set: cap entries, -1 empty */
    uint32_t cap;
    int* rep;            /* per record: the record its word is counted under, -1 for empty */
    int* head;           /* per representative: its last duplicate, -1 */
    int* chain;          /* per duplicate: the next duplicate of its word, -1 */
    uint32_t m, r;       /* slots, displacement buckets */
    int* owner;          /* m slots: representative, -1 empty */
    uint32_t* bsize;     /* r: words per bucket */
    int* bkeys;          /* r x GREP_MAX_BUCKET: each bucket's representatives */
    uint16_t* dsp;       /* r displacements */
    unsigned long long* hset; /* duplicate-hash check: cap entries, ~0 empty */
    uint32_t* fail;      /* [0] set while the current seed fails; [1] the seed that succeeded;
                            [2] the current seed's largest bucket */
    uint32_t seed0, n_seeds; /* seeds tried: seed0 .. seed0 + n_seeds - 1 */
    grep_hashk hk;       /* filled by the host from the seed that succeeded */
    /* the image */
    uint16_t* tags;
    uint16_t* disp;
    uint4* rec_lo;
    uint4* rec_hi;
    uint32_t* slot_word;
    int32_t* next_dup;
};

static __global__ void k_tb_keys(TbDev T) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= T.n) return;
    const uint4* r = (const uint4*)(T.dict + (size_t)w * 32);
    const uint4 a = r[0], b = r[1];
    uint32_t k[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    /* length: bytes before the first NUL; key bytes after it are zero */
    int len = 32;
    for (int i = 0; i < 8 && len == 32; i++) {
        const uint32_t x = k[i];
        for (int j = 0; j < 4; j++)
            if (((x >> (8 * j)) & 0xFFu) == 0u) {
                len = 4 * i + j;
                break;
            }
    }
    for (int i = 0; i < 8; i++) {
        const int kb = len * 8 - 32 * i;
        k[i] &= kb >= 32 ? 0xFFFFFFFFu : (kb <= 0 ? 0u : ((1u << kb) - 1u));
    }
    T.klo[w] = make_uint4(k[0], k[1], k[2], k[3]);
    T.khi[w] = make_uint4(k[4], k[5], k[6], k[7]);
    T.len[w] = len;
    T.head[w] = -1;
    T.chain[w] = -1;
}

__device__ __forceinline__ bool tb_same(const TbDev& T, int a, int b) {
    if (T.len[a] != T.len[b]) return false;
    const uint4 x = T.klo[a], y = T.klo[b], u = T.khi[a], v = T.khi[b];
    return x.x == y.x && x.y == y.y && x.z == y.z && x.w == y.w && u.x == v.x && u.y == v.y && u.z == v.z && u.w == v.w;
}

/* the first record of each distinct word to claim its set entry becomes the
 * word's representative; the others are its duplicates.  The set is probed
 * by a hash of the key alone (not the seeded one), so it runs once. */
static __global__ void k_tb_dedupe(TbDev T) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= T.n) return;
    if (T.len[w] == 0) {
        T.rep[w] = -1;
        return;
    }
    const uint4 x = T.klo[w], y = T.khi[w];
    const uint32_t hs = (x.x * 0x9E3779B1u) ^ (x.y * 0x85EBCA77u) ^ (x.z * 0xC2B2AE3Du) ^ (x.w * 0x27D4EB2Fu) ^
                        (y.x * 0x165667B1u) ^ (y.y * 0xD3A2646Du) ^ (y.z * 0xFD7046C5u) ^ (y.w * 0xB55A4F09u);
    uint32_t i = grep_h1(hs) & (T.cap - 1u);
    for (uint32_t probe = 0; probe < T.cap; probe++, i = (i + 1u) & (T.cap - 1u)) {
        int cur = T.set[i];
        if (cur < 0) {
            cur = atomicCAS(&T.set[i], -1, w);
            if (cur < 0) {
                T.rep[w] = w;
                return;
            }
        }
        if (tb_same(T, cur, w)) {
            T.rep[w] = cur;
            return;
        }
    }
    T.rep[w] = w; /* unreachable: the set has twice the records' entries */
}

static __global__ void k_tb_chains(TbDev T) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= T.n) return;
    const int r = T.rep[w];
    if (r >= 0 && r != w) T.chain[w] = atomicExch(&T.head[r], w);
}

/* The seeded part of the device build, in one cooperative launch (grid-wide
 * syncs between the steps).  For each seed in turn, until one succeeds:
 *   1. every distinct word's hash under the seed's multipliers;
 *   2. a check that no two distinct words share a 32-bit hash (no
 *      displacement could separate them), through a set keyed by the hash,
 *      and the words grouped by bucket (fixed lists of GREP_MAX_BUCKET);
 *   3. the displacement search: size classes from the largest bucket size
 *      down to 1, so large buckets are placed while the table is emptiest
 *      (as in the sequential build); inside a class every warp takes
 *      buckets in turn.  A bucket's warp tests 32 displacements per round
 *      (lane l tries base + l, loading the owners of all the bucket's
 *      candidate slots at once); for the first displacement that fits,
 *      lanes 0..z-1 claim the z slots by CAS together and undo their claims
 *      if any lost a race to another bucket.
 * On success fail[1] holds the seed, T.owner the slot of every word and
 * T.dsp the displacements; fail[0] stays set if every seed failed. */
static __global__ void __launch_bounds__(256) k_tb_search(TbDev T) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const uint32_t gw = tid >> 5, nw = nth >> 5;
    for (uint32_t sd = T.seed0; sd < T.seed0 + T.n_seeds; sd++) {
        grep_hashk hk;
        grep_hash_seed(sd, &hk);
        if (tid == 0) {
            T.fail[0] = 0u;
            T.fail[2] = 0u;
        }
        for (uint32_t b = tid; b < T.r; b += nth) {
            T.bsize[b] = 0u;
            T.dsp[b] = 0;
        }
        for (uint32_t sl = tid; sl < T.m; sl += nth) T.owner[sl] = -1;
        for (uint32_t i = tid; i < T.cap; i += nth) T.hset[i] = ~0ull;
        for (int w = (int)tid; w < T.n; w += (int)nth)
            if (T.rep[w] == w) {
                const uint4 x = T.klo[w], y = T.khi[w];
                const uint32_t k[8] = {x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
                T.h1[w] = grep_h1(grep_mix(&hk, k, T.len[w]));
            }
        grid.sync();
        for (int w = (int)tid; w < T.n; w += (int)nth)
            if (T.rep[w] == w) {
                const uint32_t h = T.h1[w];
                const unsigned long long e = ((unsigned long long)h << 32) | (uint32_t)w;
                for (uint32_t i = h & (T.cap - 1u), probe = 0; probe < T.cap; probe++, i = (i + 1u) & (T.cap - 1u)) {
                    const unsigned long long cur = atomicCAS(&T.hset[i], ~0ull, e);
                    if (cur == ~0ull) break;
                    if ((uint32_t)(cur >> 32) == h) {
                        atomicOr(&T.fail[0], 1u);
                        break;
                    }
                }
                const uint32_t b = grep_bucket(h, T.r);
                const uint32_t i = atomicAdd(&T.bsize[b], 1u);
                if (i < GREP_MAX_BUCKET) T.bkeys[(size_t)b * GREP_MAX_BUCKET + i] = w;
                else atomicOr(&T.fail[0], 1u);
                atomicMax(&T.fail[2], i + 1u); /* the largest bucket */
            }
        grid.sync();
        bool failed = *(volatile uint32_t*)&T.fail[0] != 0u;
        const int zmax = (int)min(*(volatile uint32_t*)&T.fail[2], (uint32_t)GREP_MAX_BUCKET);
        for (int z = zmax; z >= 1 && !failed; z--) {
            for (uint32_t b = gw; b < T.r; b += nw) {
                if (T.bsize[b] != (uint32_t)z) continue;
                const int* keys = T.bkeys + (size_t)b * GREP_MAX_BUCKET;
                uint32_t hh[GREP_MAX_BUCKET];
                for (int i = 0; i < z; i++) hh[i] = T.h1[keys[i]];
                const int mykey = lane < (uint32_t)z ? keys[lane] : -1;
                const uint32_t myh = lane < (uint32_t)z ? hh[lane] : 0u;
                uint32_t found = 0xFFFFFFFFu;
                for (uint32_t base = 0; base < 65536u && found == 0xFFFFFFFFu; base += 32u) {
                    const uint32_t d = base + lane;
                    uint32_t sl[GREP_MAX_BUCKET];
                    bool ok = true;
                    for (int i = 0; i < z; i++) {
                        sl[i] = grep_slot(hh[i], d, T.m);
                        for (int q = 0; q < i; q++) ok = ok && sl[q] != sl[i];
                    }
                    /* owners of all candidate slots: independent loads, 8 in flight */
                    for (int i0 = 0; i0 < z; i0 += 8) {
                        int o[8];
#pragma unroll
                        for (int j = 0; j < 8; j++) o[j] = i0 + j < z ? ((volatile int*)T.owner)[sl[i0 + j]] : -1;
#pragma unroll
                        for (int j = 0; j < 8; j++) ok = ok && o[j] < 0;
                    }
                    unsigned cand = __ballot_sync(0xFFFFFFFFu, ok);
                    while (cand) {
                        const int l = __ffs(cand) - 1;
                        cand &= cand - 1u;
                        const uint32_t dd = base + (uint32_t)l;
                        bool mine = false;
                        if (lane < (uint32_t)z) mine = atomicCAS(&T.owner[grep_slot(myh, dd, T.m)], -1, mykey) == -1;
                        const unsigned lost = __ballot_sync(0xFFFFFFFFu, lane < (uint32_t)z && !mine);
                        if (!lost) {
                            found = dd;
                            break;
                        }
                        if (mine) atomicExch(&T.owner[grep_slot(myh, dd, T.m)], -1);
                    }
                }
                if (lane == 0) {
                    if (found == 0xFFFFFFFFu) atomicOr(&T.fail[0], 1u);
                    else T.dsp[b] = (uint16_t)found;
                }
            }
            grid.sync();
            failed = *(volatile uint32_t*)&T.fail[0] != 0u;
        }
        if (!failed) {
            if (tid == 0) T.fail[1] = sd;
            return;
        }
        grid.sync(); /* every thread has read the flag before the next seed clears it */
    }
}

static __global__ void k_tb_image(TbDev T) {
    const uint32_t sl = blockIdx.x * blockDim.x + threadIdx.x;
    if (sl < T.m) {
        const int w = T.owner[sl];
        if (w < 0) {
            T.tags[sl] = 0;
            T.rec_lo[sl] = make_uint4(0u, 0u, 0u, 0u);
            T.rec_hi[sl] = make_uint4(0u, 0u, 0u, 0u);
            T.slot_word[sl] = 0xFFFFFFFFu;
        } else {
            T.tags[sl] = (uint16_t)grep_tag(T.h1[w], T.len[w]);
            T.rec_lo[sl] = T.klo[w];
            T.rec_hi[sl] = T.khi[w];
            T.slot_word[sl] = (uint32_t)w;
        }
    }
    if (sl < T.r) T.disp[sl] = T.dsp[sl];
    /* duplicate chains: representative -> its duplicates -> -1 */
    if (sl < (uint32_t)T.n) T.next_dup[sl] = T.rep[sl] == (int)sl ? T.head[sl] : T.chain[sl];
}

static __global__ void k_open_files(const char* names, int n, int* fds, uint64_t* sizes, int oflags = O_GRDONLY) {
    int f = blockIdx.x;
    if (f >= n) return;
    gfs_state* S = g_gfs;
    int fd = gfsd::blk_open(S, names + (size_t)f * GFS_NAME_MAX, oflags);
    if (threadIdx.x == 0) {
        fds[f] = fd;
        sizes[f] = fd >= 0 ? gfsd::ld_rlx64(&S->files[fd].size) : 0;
    }
}

/* counts matrix -> the caller's host memory, written by the SMs through the
 * host page tables: 16-byte stores where the destination allows, then the
 * 4-byte tail */
static __global__ void __launch_bounds__(256) k_counts_out(const uint32_t* __restrict__ src, uint32_t* dst, size_t n) {
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (size_t)gridDim.x * blockDim.x;
    size_t done = 0;
    if (((uintptr_t)dst & 15u) == 0u) {
        const size_t n16 = n / 4u;
        const uint4* s4 = (const uint4*)src;
        uint4* d4 = (uint4*)dst;
        for (size_t i = tid; i < n16; i += nth) d4[i] = __ldg(s4 + i);
        done = n16 * 4u;
    }
    for (size_t i = done + tid; i < n; i += nth) dst[i] = __ldg(src + i);
}

static __global__ void k_close_files(const int* fds, int n, int* rcs) {
    int f = blockIdx.x;
    if (f >= n) return;
    int fd = fds[f];
    int r = fd >= 0 ? gfsd::blk_close(g_gfs, fd) : 0;
    if (threadIdx.x == 0) rcs[f] = r;
}

namespace {

static_assert(__BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__, "record keys are little-endian words, as on the device");

/* Key words of a 32-byte record (bytes up to its first NUL, zero padded). */
void rec_key(const uint8_t* rec, uint32_t k[8], int* len) {
    const void* z = memchr(rec, 0, 32);
    const int l = z ? (int)((const uint8_t*)z - rec) : 32;
    memset(k, 0, 32);
    memcpy(k, rec, (size_t)l);
    *len = l;
}

/* Host workspace of table builds, kept across plans so a build touches no
 * freshly mapped memory; one build at a time. */
struct BuildWs {
    struct Key {
        uint32_t k[8];
        uint32_t h1;
        int len;
    };
    std::mutex mu;
    std::vector<Key> key;
    std::vector<int> uniq, last, seen, slot_of, bkeys;
    std::vector<uint32_t> bstart, bfill, order;
    std::vector<uint16_t> disp;
    std::vector<int32_t> next_dup;
    uint32_t m = 0, r = 0;
    grep_hashk hk{};
};
BuildWs g_ws;

/* Host build of the table (the fallback of the device build, and the build
 * a session with GFS_CFG_HOST_TABLE asks for): the same geometry, hashes
 * and displacement search as k_tb_search, one bucket at a time, largest
 * first.  Result in W: m, r, hk, slot_of (slot -> first record of its word,
 * -1 empty), disp, next_dup. */
bool build_table(const uint8_t* dict, int n_words, BuildWs& W) {
    const size_t nw = n_words > 0 ? (size_t)n_words : 1u;
    auto& key = W.key;
    key.resize(nw);
    W.uniq.clear();
    W.uniq.reserve(nw);
    W.last.assign(nw, -1);
    W.next_dup.assign(nw, -1);
    /* duplicates: open addressing on a hash of the key, exact key compare */
    size_t cap = 16;
    while (cap < 2 * nw) cap <<= 1;
    W.seen.assign(cap, -1);
    for (int w = 0; w < n_words; w++) {
        BuildWs::Key& kw = key[(size_t)w];
        rec_key(dict + (size_t)w * 32, kw.k, &kw.len);
        if (kw.len == 0) continue;
        uint32_t hs = 0;
        for (int i = 0; i < 8; i++) hs ^= kw.k[i] * (0x9E3779B1u + 0x3C6EF372u * (uint32_t)i);
        for (size_t i = grep_h1(hs) & (cap - 1);; i = (i + 1) & (cap - 1)) {
            const int u = W.seen[i];
            if (u < 0) {
                W.seen[i] = w;
                W.uniq.push_back(w);
                W.last[(size_t)w] = w;
                break;
            }
            const BuildWs::Key& ku = key[(size_t)u];
            if (ku.len == kw.len && memcmp(ku.k, kw.k, sizeof kw.k) == 0) {
                W.next_dup[(size_t)W.last[(size_t)u]] = w;
                W.last[(size_t)u] = w;
                break;
            }
        }
    }
    uint32_t m0, r;
    grep_geometry((uint32_t)n_words, &m0, &r);
    for (uint32_t seed = 0; seed < 16; seed++) {
        const uint32_t m = m0 + m0 / 16u * (seed / 8u);
        grep_hash_seed(seed, &W.hk);
        for (int w : W.uniq) key[(size_t)w].h1 = grep_h1(grep_mix(&W.hk, key[(size_t)w].k, key[(size_t)w].len));
        /* words grouped by bucket */
        W.bstart.assign((size_t)r + 1, 0u);
        for (int w : W.uniq) W.bstart[grep_bucket(key[(size_t)w].h1, r) + 1]++;
        for (uint32_t b = 0; b < r; b++) W.bstart[b + 1] += W.bstart[b];
        W.bfill.assign(W.bstart.begin(), W.bstart.end() - 1);
        W.bkeys.resize(W.uniq.size() + 1);
        for (int w : W.uniq) W.bkeys[W.bfill[grep_bucket(key[(size_t)w].h1, r)]++] = w;
        /* buckets by decreasing size */
        W.order.resize(r);
        for (uint32_t b = 0; b < r; b++) W.order[b] = b;
        std::stable_sort(W.order.begin(), W.order.end(), [&](uint32_t x, uint32_t y) {
            return W.bstart[x + 1] - W.bstart[x] > W.bstart[y + 1] - W.bstart[y];
        });
        W.slot_of.assign(m, -1);
        W.disp.assign(r, 0);
        bool ok = true;
        for (uint32_t b : W.order) {
            const uint32_t z = W.bstart[b + 1] - W.bstart[b];
            if (z == 0) break;
            if (z > GREP_MAX_BUCKET) { ok = false; break; }
            const int* ks = W.bkeys.data() + W.bstart[b];
            uint32_t sl[GREP_MAX_BUCKET];
            for (uint32_t i = 0; i < z && ok; i++)
                for (uint32_t q = 0; q < i; q++)
                    if (key[(size_t)ks[q]].h1 == key[(size_t)ks[i]].h1) ok = false;
            uint32_t d = 0;
            for (; ok && d < 65536u; d++) {
                bool fit = true;
                for (uint32_t i = 0; i < z && fit; i++) {
                    sl[i] = grep_slot(key[(size_t)ks[i]].h1, d, m);
                    fit = W.slot_of[sl[i]] < 0;
                    for (uint32_t q = 0; q < i && fit; q++) fit = sl[q] != sl[i];
                }
                if (fit) break;
            }
            if (!ok || d >= 65536u) { ok = false; break; }
            for (uint32_t i = 0; i < z; i++) W.slot_of[sl[i]] = ks[i];
            W.disp[b] = (uint16_t)d;
        }
        if (!ok) continue;
        W.m = m;
        W.r = r;
        return true;
    }
    return false;
}

} // namespace

struct gfs_grep {
    gfs_ctx* ctx = nullptr;
    int n_files = 0, n_words = 0;
    uint32_t m = 0, r = 0; /* table slots, displacement buckets */
    GrepDev dev{};
    void* dmem = nullptr; /* one allocation for everything */
    std::vector<uint64_t> sizes;
    bool smem = true;
    size_t smem_bytes = 0;
    int sms = 0;
    uint32_t last_status[2] = {0, 0};
    long long build_us = 0, open_us = 0; /* host time of the table build / of opening the files */
    /* batched run: captured once per grid size, replayed */
    cudaGraphExec_t batch_graph = nullptr;
    int batch_ctas = 0;
    /* the bytes the reference's chunk walk reads twice (k_grep_tail): the
     * first run walks the files on host threads while its scan runs */
    std::vector<int> hfds;              /* device file slot of each file */
    uint64_t* tail = nullptr;           /* per file: start, its size if none, ~0 if unreadable;
                                           mapped pinned memory, read by k_grep_tail */
    std::atomic<int> tail_next{0};      /* next file to walk */
    bool tail_done = false;
    int tail_files = 0, tail_err = 0;   /* files with such bytes; -errno */
};

/* Pages per window so that all CTAs' pinned windows (two each) fit in half
 * the pool; the kernel halves it further if frames still run short. */
static void set_window(gfs_grep* g, int n_ctas) {
    uint32_t frames = gfs_num_frames(g->ctx);
    uint64_t per = (uint64_t)frames / 2u / (uint64_t)(n_ctas > 0 ? n_ctas : 1);
    g->dev.win_pages = per > GR_WIN ? GR_WIN : (uint32_t)(per ? per : 1u); /* the kernel raises it to one chunk */
}

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

static uint64_t host_us() {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (uint64_t)ts.tv_sec * 1000000ull + (uint64_t)ts.tv_nsec / 1000ull;
}

/* Device layout of a plan: the table image and the file names first, then
 * what the device fills or the host adds later.  Tags and displacements are
 * zero padded to their shared-memory sizes (the scan copies them whole). */
struct PlanLayout {
    size_t o_tbl, o_disp, o_recs, o_sw, o_nd, o_names, o_cnt, o_fds, o_sz, o_pf, o_fl, o_st, o_fo, o_fn, o_xxh,
        o_maps, total;
};
static PlanLayout plan_layout(uint32_t m, uint32_t r, int n_words, int n_files) {
    PlanLayout L;
    L.o_tbl = 0;
    L.o_disp = align_up(L.o_tbl + grep_tag_smem(m), 256);
    L.o_recs = align_up(L.o_disp + grep_disp_smem(r), 256);
    L.o_sw = align_up(L.o_recs + (size_t)m * 32, 256);
    L.o_nd = align_up(L.o_sw + (size_t)m * 4, 256);
    L.o_names = align_up(L.o_nd + (size_t)n_words * 4 + 4, 256);
    L.o_cnt = align_up(L.o_names + (size_t)n_files * GFS_NAME_MAX, 256);
    L.o_fds = align_up(L.o_cnt + (size_t)n_words * n_files * 4 + 4, 256);
    L.o_sz = align_up(L.o_fds + (size_t)n_files * 4, 256);
    L.o_pf = align_up(L.o_sz + (size_t)n_files * 8, 256);
    L.o_fl = align_up(L.o_pf + (size_t)(n_files + 1) * 8, 256);
    L.o_st = align_up(L.o_fl + (size_t)n_files * 4, 256);
    L.o_fo = align_up(L.o_st + 64, 256);
    L.o_fn = align_up(L.o_fo + (size_t)n_files * 4, 256);
    L.o_xxh = align_up(L.o_fn + 64, 256);
    L.o_maps = align_up(L.o_xxh + (size_t)n_files * 8, 256);
    L.total = align_up(L.o_maps + (size_t)n_files * 8, 256);
    return L;
}

/* ---------------- the bytes the reference's walk reads twice ---------------- */
static inline bool host_alpha(uint8_t c) { return (uint32_t)(c | 32u) - 97u < 26u || c == 95u; }

/* The reference's chunk walk over one file (grep_text_gpu.cu:298-318):
 * windows of 16384 + 32 bytes; a window short of the end moves the cursor
 * 16384 bytes plus the letters that begin its 32-byte halo (find_overlap,
 * :89-101), the last window 16384 bytes as well, so when the last window is
 * longer than 16384 bytes the loop goes round once more and reads the bytes
 * past the cursor again.  Returns where those bytes start, `size` when there
 * are none, or UINT64_MAX when a halo could not be read.  halo(off, h) reads
 * the 32 bytes at off (always inside the file); ahead(off, n) may prefetch
 * bytes that a later step reads. */
template <class Halo, class Ahead>
static uint64_t walk_tail_start(uint64_t size, Halo&& halo, Ahead&& ahead) {
    const uint64_t W = 16384u, H = 32u;
    uint64_t c = 0;
    while (size - c >= W + H) {
        /* the cursor four windows on is in [c + 4W, c + 4(W + H)], so its
         * halo is in [c + 5W, c + 5W + 5H) */
        ahead(c + 5u * W, 5u * H);
        uint8_t h[32];
        if (!halo(c + W, h)) return UINT64_MAX;
        uint64_t ov = 0;
        while (ov < H && host_alpha(h[ov])) ov++;
        c += W + ov;
    }
    return size - c > W ? c + W : size;
}

/* the walk over bytes in host memory (a file's mapping) */
static uint64_t tail_start_mem(const uint8_t* b, uint64_t size) {
    return walk_tail_start(
        size,
        [&](uint64_t off, uint8_t* h) {
            memcpy(h, b + off, 32);
            return true;
        },
        [&](uint64_t off, uint64_t n) {
            const uint64_t e = off + n < size ? off + n : size;
            for (uint64_t a = off & ~(uint64_t)63; a < e; a += 64) __builtin_prefetch(b + a);
        });
}

/* the walk over an open file slot: its host mapping, else pread */
static uint64_t tail_start_slot(gfs_ctx* ctx, uint32_t slot, uint64_t size) {
    const uint8_t* base = nullptr;
    unsigned long long len = 0;
    if (gfs__slot_map_host(ctx, slot, &base, &len) > 0 && base && len >= size) return tail_start_mem(base, size);
    return walk_tail_start(
        size, [&](uint64_t off, uint8_t* h) { return gfs__slot_pread(ctx, slot, h, 32, off) == 32; },
        [](uint64_t, uint64_t) {});
}

static void tail_walk_files(gfs_grep* g) {
    for (int f; (f = g->tail_next.fetch_add(1)) < g->n_files;)
        g->tail[(size_t)f] = tail_start_slot(g->ctx, (uint32_t)g->hfds[(size_t)f], g->sizes[(size_t)f]);
}

/* Walks every file once, on up to 4 host threads and the calling one (a
 * quarter of the cores at most: the host workers serving the scan's page
 * fills keep the rest), the first time a run asks, after it has launched
 * its scan, so the walk overlaps the scan.  Returns the number of files with bytes read twice,
 * or -errno.  It makes no CUDA call: it runs while the plan's kernels may be
 * waiting on the host workers, and a call that waits on the stream could
 * hold them up. */
static int tail_finish(gfs_grep* g) {
    if (!g->tail_done) {
        g->tail_next.store(0);
        std::vector<std::thread> th;
        unsigned nt = std::thread::hardware_concurrency() / 4u;
        nt = nt > 4u ? 4u : nt;
        if (nt + 1u > (unsigned)g->n_files) nt = g->n_files > 1 ? (unsigned)g->n_files - 1u : 0u;
        try {
            for (unsigned i = 0; i < nt; i++) th.emplace_back(tail_walk_files, g);
        } catch (...) {
            /* fewer threads: this one walks what is left */
        }
        tail_walk_files(g);
        for (auto& t : th) t.join();
        g->tail_done = true;
        int n = 0;
        for (int i = 0; i < g->n_files && !g->tail_err; i++) {
            const uint64_t t = g->tail[(size_t)i];
            if (t == UINT64_MAX) g->tail_err = -GFS_EIO;
            else if (t < g->sizes[(size_t)i]) n++;
        }
        g->tail_files = n;
    }
    return g->tail_err ? g->tail_err : g->tail_files;
}

extern "C" uint64_t gfs__grep_tail_start(const uint8_t* bytes, uint64_t size) { return tail_start_mem(bytes, size); }

/* Device build of the dictionary table (the dictionary's n_words records
 * are in pinned host memory at hdict; flag is 8 spare pinned bytes).  On
 * success returns true and leaves the build state (geometry, seed) in *T
 * and its memory in *tmp; the caller runs k_tb_image into the plan memory
 * and frees *tmp.  false: every seed failed, or the device could not run
 * the cooperative search (*tmp freed); the caller builds on the host. */
static bool device_table(gfs_ctx* ctx, cudaStream_t s, const uint8_t* hdict, uint32_t* flag, int n_words,
                         TbDev* T, void** tmp) {
    const size_t n = (size_t)(n_words > 0 ? n_words : 1);
    uint32_t cap = 16;
    while (cap < 2 * n) cap <<= 1;
    uint32_t m0, r;
    grep_geometry((uint32_t)n_words, &m0, &r);
    const uint32_t m_max = m0 + m0 / 16u * 2u;
    const size_t o_dict = 0, o_klo = align_up(n * 32, 256), o_khi = align_up(o_klo + n * 16, 256),
                 o_h1 = align_up(o_khi + n * 16, 256), o_len = align_up(o_h1 + n * 4, 256),
                 o_rep = align_up(o_len + n * 4, 256), o_head = align_up(o_rep + n * 4, 256),
                 o_nd = align_up(o_head + n * 4, 256), o_set = align_up(o_nd + n * 4, 256),
                 o_hs = align_up(o_set + (size_t)cap * 4, 256), o_own = align_up(o_hs + (size_t)cap * 8, 256),
                 o_bsz = align_up(o_own + (size_t)m_max * 4, 256), o_bk = align_up(o_bsz + (size_t)r * 4, 256),
                 o_dsp = align_up(o_bk + (size_t)r * GREP_MAX_BUCKET * 4, 256),
                 o_fail = align_up(o_dsp + (size_t)r * 2, 256), total = o_fail + 256;
    uint8_t* mem = (uint8_t*)gfs__dev_alloc(ctx, total, s);
    *tmp = mem;
    if (!mem) return false;
    TbDev& D = *T;
    D.dict = mem + o_dict;
    D.n = n_words;
    D.klo = (uint4*)(mem + o_klo);
    D.khi = (uint4*)(mem + o_khi);
    D.h1 = (uint32_t*)(mem + o_h1);
    D.len = (int*)(mem + o_len);
    D.rep = (int*)(mem + o_rep);
    D.head = (int*)(mem + o_head);
    D.set = (int*)(mem + o_set);
    D.cap = cap;
    D.chain = (int*)(mem + o_nd);
    D.hset = (unsigned long long*)(mem + o_hs);
    D.owner = (int*)(mem + o_own);
    D.bsize = (uint32_t*)(mem + o_bsz);
    D.bkeys = (int*)(mem + o_bk);
    D.dsp = (uint16_t*)(mem + o_dsp);
    D.fail = (uint32_t*)(mem + o_fail);
    D.r = r;
    const int nt = 256, gw = (n_words + nt - 1) / nt;
    /* the cooperative search: at most four 256-thread blocks per SM, as many
     * as fit at once */
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tb_search, nt, 0);
    const int blocks = sms * (per_sm < 4 ? per_sm : 4);
    cudaMemsetAsync(D.fail, 0, 8, s);
    if (n_words > 0) {
        cudaMemcpyAsync(mem + o_dict, hdict, (size_t)n_words * 32, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(D.set, 0xFF, (size_t)cap * 4, s);
        k_tb_keys<<<gw, nt, 0, s>>>(D);
        k_tb_dedupe<<<gw, nt, 0, s>>>(D);
        k_tb_chains<<<gw, nt, 0, s>>>(D);
    }
    /* 8 seeds at the base size, then 4 at each of two larger tables */
    const uint32_t plan[3][2] = {{0u, 8u}, {8u, 4u}, {12u, 4u}};
    for (int a = 0; a < 3 && blocks > 0; a++) {
        D.m = m0 + m0 / 16u * (uint32_t)a;
        D.seed0 = plan[a][0];
        D.n_seeds = plan[a][1];
        void* args[] = {&D};
        if (cudaLaunchCooperativeKernel((const void*)k_tb_search, dim3((unsigned)blocks), dim3(nt), args, 0, s) !=
            cudaSuccess)
            break;
        cudaMemcpyAsync(flag, D.fail, 8, cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) break;
        if (flag[0] == 0u) {
            grep_hash_seed(flag[1], &D.hk);
            return true;
        }
    }
    cudaGetLastError();
    gfs__dev_free(ctx, mem, s);
    *tmp = nullptr;
    return false;
}

extern "C" {

void gfs__preload_grep() {
    cudaFuncAttributes a;
    cudaFuncGetAttributes(&a, k_grep_scan<true, false, false>);
    cudaFuncGetAttributes(&a, k_grep_scan<false, false, false>);
    cudaFuncGetAttributes(&a, k_grep_scan<true, true, false>);
    cudaFuncGetAttributes(&a, k_grep_scan<false, true, false>);
    cudaFuncGetAttributes(&a, k_grep_scan<true, false, true>);
    cudaFuncGetAttributes(&a, k_grep_scan<false, false, true>);
    cudaFuncGetAttributes(&a, k_serve);
    cudaFuncGetAttributes(&a, k_grep_fixup);
    cudaFuncGetAttributes(&a, k_grep_tail);
    cudaFuncGetAttributes(&a, k_counts_out);
    cudaFuncGetAttributes(&a, k_open_files);
    cudaFuncGetAttributes(&a, k_close_files);
}

int gfs_grep_open(gfs_ctx* ctx, const char* dict_path, const char* const* paths, int n_files, gfs_grep** out) {
    *out = nullptr;
    if (n_files < 1 || !dict_path) return -GFS_EINVAL;
    for (int i = 0; i < n_files; i++)
        if (!paths[i] || strlen(paths[i]) >= GFS_NAME_MAX) return -GFS_EINVAL;
    if (gfs__activate(ctx)) return -GFS_EIO;
    for (int i = 0; i < n_files; i++) gfs__premap(ctx, paths[i]);
    int fd = open(dict_path, O_RDONLY | O_CLOEXEC);
    if (fd < 0) return -errno;
    struct stat st;
    if (fstat(fd, &st) != 0) { const int e = errno; close(fd); return -e; }
    const int n_words = (int)(st.st_size / 32); /* grep_text_gpu.cu:221 */
    const size_t dict_bytes = (size_t)n_words * 32;
    cudaStream_t s = (cudaStream_t)gfs_kernel_stream(ctx);
    /* the dictionary goes straight into the session's pinned buffer */
    const size_t names_bytes = (size_t)n_files * GFS_NAME_MAX;
    uint8_t* hb = (uint8_t*)gfs__host_bounce(ctx, align_up(dict_bytes, 256) + 256 + names_bytes);
    if (!hb) { close(fd); return -GFS_ENOMEM; }
    size_t got = 0;
    while (got < dict_bytes) {
        ssize_t r = pread(fd, hb + got, dict_bytes - got, (off_t)got);
        if (r <= 0) break;
        got += (size_t)r;
    }
    close(fd);
    if (got < dict_bytes) return -GFS_EIO;
    gfs_grep* g = new gfs_grep();
    g->ctx = ctx;
    g->n_files = n_files;
    g->n_words = n_words;
    int dev = 0, sms = 0, maxsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t fixed = (size_t)GR_STAGES * GR_STAGE + (size_t)GR_CONS * GR_WSCR + 256;
    const uint64_t t_build = host_us();
    TbDev T{};
    void* tmp = nullptr;
    const bool on_dev = !(gfs__config_flags(ctx) & GFS_CFG_HOST_TABLE) &&
                        device_table(ctx, s, hb, (uint32_t*)(hb + align_up(dict_bytes, 256)), n_words, &T, &tmp);
    std::unique_lock<std::mutex> lk(g_ws.mu, std::defer_lock);
    uint32_t m, r;
    grep_hashk hk;
    if (on_dev) {
        m = T.m;
        r = T.r;
        hk = T.hk;
    } else {
        /* the device search gave up (or the session asked for it): build
         * on the host */
        lk.lock();
        if (!build_table(hb, n_words, g_ws)) { delete g; return -GFS_ENOMEM; }
        m = g_ws.m;
        r = g_ws.r;
        hk = g_ws.hk;
    }
    g->m = m;
    g->r = r;
    const PlanLayout L = plan_layout(m, r, n_words, n_files);
    const size_t o_tbl = L.o_tbl, o_disp = L.o_disp, o_recs = L.o_recs, o_sw = L.o_sw, o_nd = L.o_nd,
                 o_names = L.o_names, o_cnt = L.o_cnt, o_fds = L.o_fds, o_sz = L.o_sz, o_pf = L.o_pf, o_fl = L.o_fl,
                 o_st = L.o_st, o_fo = L.o_fo, o_fn = L.o_fn, o_xxh = L.o_xxh, o_maps = L.o_maps, total = L.total;
    g->dmem = gfs__dev_alloc(ctx, total, s);
    if (!g->dmem || !(hb = (uint8_t*)gfs__host_bounce(ctx, tmp ? names_bytes : o_cnt))) {
        gfs__dev_free(ctx, tmp, s);
        gfs__dev_free(ctx, g->dmem, s);
        delete g;
        return -GFS_ENOMEM;
    }
    uint8_t* b = (uint8_t*)g->dmem;
    cudaMemsetAsync(b + o_cnt, 0, total - o_cnt, s);
    if (tmp) {
        /* the device-built image (tags and displacements zero padded), then
         * the names */
        cudaMemsetAsync(b, 0, o_recs, s);
        T.tags = (uint16_t*)(b + o_tbl);
        T.disp = (uint16_t*)(b + o_disp);
        T.rec_lo = (uint4*)(b + o_recs);
        T.rec_hi = T.rec_lo + m;
        T.slot_word = (uint32_t*)(b + o_sw);
        T.next_dup = (int32_t*)(b + o_nd);
        const uint32_t items = m > (uint32_t)n_words ? m : (uint32_t)n_words;
        k_tb_image<<<(items + 255) / 256, 256, 0, s>>>(T);
        gfs__dev_free(ctx, tmp, s);
        memset(hb, 0, names_bytes);
        for (int i = 0; i < n_files; i++) memcpy(hb + (size_t)i * GFS_NAME_MAX, paths[i], strlen(paths[i]));
        cudaMemcpyAsync(b + o_names, hb, names_bytes, cudaMemcpyHostToDevice, s);
    } else {
        /* the host-built image: slot tags, displacements, record bytes
         * 0..15 of every slot, then bytes 16..31, first record of each
         * slot, duplicate chains; names */
        BuildWs& W = g_ws;
        memset(hb, 0, o_cnt);
        uint16_t* tags = (uint16_t*)(hb + o_tbl);
        uint32_t* lo = (uint32_t*)(hb + o_recs);
        uint32_t* hi = lo + (size_t)m * 4;
        uint32_t* sw = (uint32_t*)(hb + o_sw);
        for (size_t sl = 0; sl < m; sl++) {
            const int w = W.slot_of[sl];
            if (w < 0) {
                sw[sl] = 0xFFFFFFFFu;
                continue;
            }
            const BuildWs::Key& kw = W.key[(size_t)w];
            tags[sl] = (uint16_t)grep_tag(kw.h1, kw.len);
            memcpy(lo + sl * 4, kw.k, 16);
            memcpy(hi + sl * 4, kw.k + 4, 16);
            sw[sl] = (uint32_t)w;
        }
        memcpy(hb + o_disp, W.disp.data(), (size_t)r * 2);
        if (n_words) memcpy(hb + o_nd, W.next_dup.data(), (size_t)n_words * 4);
        for (int i = 0; i < n_files; i++) memcpy(hb + o_names + (size_t)i * GFS_NAME_MAX, paths[i], strlen(paths[i]));
        cudaMemcpyAsync(b, hb, o_cnt, cudaMemcpyHostToDevice, s);
        lk.unlock();
    }
    g->build_us = (long long)(host_us() - t_build);
    GrepDev& d = g->dev;
    d.n_files = n_files;
    d.n_words = g->n_words;
    d.fds = (const int*)(b + o_fds);
    d.sizes = (const uint64_t*)(b + o_sz);
    d.chunk_prefix = (const uint64_t*)(b + o_pf);
    d.m = m;
    d.r = r;
    d.hk = hk;
    d.tags = (const uint16_t*)(b + o_tbl);
    d.disp = (const uint16_t*)(b + o_disp);
    d.rec_lo = (const uint4*)(b + o_recs);
    d.rec_hi = d.rec_lo + m;
    d.slot_word = (const uint32_t*)(b + o_sw);
    d.next_dup = (const int32_t*)(b + o_nd);
    d.counts = (uint32_t*)(b + o_cnt);
    d.long_flags = (uint32_t*)(b + o_fl);
    d.status = (uint32_t*)(b + o_st);
    d.file_order = (const int*)(b + o_fo);
    d.file_next = (uint32_t*)(b + o_fn);
    d.xxh = (unsigned long long*)(b + o_xxh);
    d.maps = (const uint64_t*)(b + o_maps);
    const uint64_t t_open = host_us();
    k_open_files<<<n_files, 128, 0, s>>>((const char*)(b + o_names), n_files, (int*)d.fds, (uint64_t*)d.sizes);
    /* slots and sizes back through the pinned buffer (the image copy before
     * the kernel on this stream is done with it by then) */
    int* fds = (int*)hb;
    uint64_t* szs = (uint64_t*)(hb + align_up((size_t)n_files * 4, 64));
    cudaMemcpyAsync(fds, d.fds, (size_t)n_files * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(szs, d.sizes, (size_t)n_files * 8, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) { gfs_grep_close(g); return -GFS_EIO; }
    g->open_us = (long long)(host_us() - t_open);
    g->sizes.assign(szs, szs + n_files);
    g->hfds.assign(fds, fds + n_files);
    for (int i = 0; i < n_files; i++)
        if (fds[i] < 0) {
            int e = fds[i];
            gfs_grep_close(g);
            return e;
        }
    {
        /* per file: its host mapping's device address (direct scans read
         * it), chunk prefix sums, and the longest-first order of batched
         * runs (LPT: the largest file bounds the run, so it starts first).
         * Copied from pageable memory: the driver stages such a copy before
         * the call returns, so the vectors may go at once and no round trip
         * to the device is needed. */
        std::vector<uint64_t> maps((size_t)n_files), pf((size_t)n_files + 1);
        std::vector<int> order((size_t)n_files);
        for (int i = 0; i < n_files; i++) {
            unsigned long long a = 0, len = 0;
            maps[(size_t)i] = gfs__slot_map(ctx, (uint32_t)fds[i], &a, &len) > 0 && len >= g->sizes[(size_t)i] ? a : 0u;
        }
        pf[0] = 0;
        for (int i = 0; i < n_files; i++) pf[(size_t)i + 1] = pf[(size_t)i] + (g->sizes[(size_t)i] + GR_CH - 1) / GR_CH;
        d.total_chunks = pf[(size_t)n_files];
        for (int i = 0; i < n_files; i++) order[(size_t)i] = i;
        std::stable_sort(order.begin(), order.end(),
                         [&](int x, int y) { return g->sizes[(size_t)x] > g->sizes[(size_t)y]; });
        if (cudaMemcpyAsync((void*)d.maps, maps.data(), (size_t)n_files * 8, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync((void*)d.chunk_prefix, pf.data(), ((size_t)n_files + 1) * 8, cudaMemcpyHostToDevice, s) !=
                cudaSuccess ||
            cudaMemcpyAsync((void*)d.file_order, order.data(), (size_t)n_files * 4, cudaMemcpyHostToDevice, s) !=
                cudaSuccess) {
            gfs_grep_close(g);
            return -GFS_EIO;
        }
    }
    /* shared memory: table (if it fits) + stages + token lists + scratch */
    g->sms = sms;
    size_t with_tbl = (size_t)grep_tag_smem(m) + grep_disp_smem(r) + grep_cnt_smem(m) + fixed;
    g->smem = with_tbl <= (size_t)maxsm;
    g->smem_bytes = g->smem ? with_tbl : fixed;
    cudaFuncSetAttribute(k_grep_scan<true, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)with_tbl);
    cudaFuncSetAttribute(k_grep_scan<false, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fixed);
    cudaFuncSetAttribute(k_grep_scan<true, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)with_tbl);
    cudaFuncSetAttribute(k_grep_scan<false, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fixed);
    cudaFuncSetAttribute(k_grep_scan<true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)with_tbl);
    cudaFuncSetAttribute(k_grep_scan<false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fixed);
    {
        /* the walk's per-file starts, where k_grep_tail reads them */
        void* th = nullptr;
        void* td = nullptr;
        if (cudaHostAlloc(&th, (size_t)n_files * 8, cudaHostAllocMapped) != cudaSuccess ||
            cudaHostGetDevicePointer(&td, th, 0) != cudaSuccess) {
            cudaGetLastError();
            if (th) cudaFreeHost(th);
            gfs_grep_close(g);
            return -GFS_ENOMEM;
        }
        g->tail = (uint64_t*)th;
        g->dev.tail_start = (const uint64_t*)td;
        for (int i = 0; i < n_files; i++) g->tail[i] = g->sizes[(size_t)i];
    }
    *out = g;
    return 0;
}

#ifdef MADV_POPULATE_WRITE
#define GFS_MADV_POPULATE_WRITE MADV_POPULATE_WRITE
#else
#define GFS_MADV_POPULATE_WRITE 23 /* Linux 5.14 */
#endif
static bool counts_out_ok(gfs_grep* g, size_t bytes);
static void counts_out(gfs_grep* g, uint32_t* host_counts, size_t bytes, cudaStream_t s);

/* One scan (+ the long-run fix-up).  host_counts: when the device may write
 * the caller's memory (counts_out_ok), the counts are written there on the
 * same stream, so the run and its counts cost one round trip; otherwise
 * nullptr. */
static int grep_run(gfs_grep* g, int n_ctas, float* kernel_ms, int direct, uint32_t* host_counts = nullptr) {
    if (!g) return -GFS_EINVAL;
    if (gfs__activate(g->ctx)) return -GFS_EIO;
    cudaStream_t s = (cudaStream_t)gfs_kernel_stream(g->ctx);
    GrepDev d = g->dev;
    cudaMemsetAsync(d.counts, 0, (size_t)g->n_words * g->n_files * 4, s);
    cudaMemsetAsync(d.long_flags, 0, (size_t)g->n_files * 4, s);
    cudaMemsetAsync(d.status, 0, 8, s);
    if (n_ctas <= 0) n_ctas = g->sms;
    set_window(g, n_ctas);
    d.win_pages = g->dev.win_pages;
    cudaEvent_t a, b;
    if (kernel_ms) {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, s);
    }
    gfs_state* S = (gfs_state*)gfs_device_state(g->ctx);
    if (direct) {
        if (g->smem) k_grep_scan<true, false, true><<<n_ctas, GR_THREADS, g->smem_bytes, s>>>(S, d);
        else k_grep_scan<false, false, true><<<n_ctas, GR_THREADS, g->smem_bytes, s>>>(S, d);
    } else {
        if (g->smem) k_grep_scan<true, false, false><<<n_ctas, GR_THREADS, g->smem_bytes, s>>>(S, d);
        else k_grep_scan<false, false, false><<<n_ctas, GR_THREADS, g->smem_bytes, s>>>(S, d);
    }
    cudaError_t le = cudaGetLastError();
    k_grep_fixup<<<g->n_files, 32, 0, s>>>(S, d);
    /* the host finishes the walk while the scan runs */
    const int n_tail = tail_finish(g);
    if (n_tail > 0) k_grep_tail<<<g->n_files, 32, 0, s>>>(S, d);
    if (kernel_ms) {
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(kernel_ms, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    if (host_counts) counts_out(g, host_counts, (size_t)g->n_words * g->n_files * 4, s);
    /* the status words come back through the session's pinned buffer with
     * the same synchronisation */
    uint32_t* status = (uint32_t*)gfs__host_bounce(g->ctx, 64);
    if (!status) return -GFS_ENOMEM;
    status[0] = status[1] = 0;
    cudaMemcpyAsync(status, d.status, 8, cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (le == cudaSuccess) le = cudaGetLastError();
    if (le != cudaSuccess || e != cudaSuccess) {
        fprintf(stderr, "gpufs_gb300: grep kernel failed: %s\n", cudaGetErrorString(le != cudaSuccess ? le : e));
        return -GFS_EIO;
    }
    g->last_status[0] = status[0];
    g->last_status[1] = status[1];
    if (status[0]) return -((status[0] & GFS_ERRB_TIMEOUT) ? GFS_ETIMEDOUT : GFS_EIO);
    return n_tail < 0 ? n_tail : 0;
}

/* Counts of up to 16 MiB go straight from the device into the caller's
 * memory when the session's device may address pageable host memory: one
 * kernel writing at link speed, no pinned staging and no host copy.  Larger
 * matrices keep the pinned path (the caller's pages may not be resident,
 * and faulting them in from the device is slower than a host copy). */
static bool counts_out_ok(gfs_grep* g, size_t bytes) {
    return bytes > 0 && bytes <= ((size_t)16 << 20) && gfs__pageable_access(g->ctx);
}
static void counts_out(gfs_grep* g, uint32_t* host_counts, size_t bytes, cudaStream_t s) {
    /* Fault the caller's pages in first, as a host write would, without
     * touching their bytes: a fresh buffer's first write from the device
     * otherwise takes a page fault per page through the host's page tables
     * (measured 0.65 ms for 2.56 MB, against 0.02 ms once the pages exist).
     * Kernels without this call still work, only slower. */
    {
        const uintptr_t pg = (uintptr_t)sysconf(_SC_PAGESIZE);
        const uintptr_t a = (uintptr_t)host_counts & ~(pg - 1u), e = ((uintptr_t)host_counts + bytes + pg - 1u) & ~(pg - 1u);
        madvise((void*)a, e - a, GFS_MADV_POPULATE_WRITE);
    }
    const size_t n = bytes / 4u;
    size_t blocks = (n / 4u + 255u) / 256u;
    const size_t cap = (size_t)(g->sms > 0 ? g->sms : 1) * 4u;
    blocks = blocks < 1u ? 1u : (blocks > cap ? cap : blocks);
    k_counts_out<<<(unsigned)blocks, 256, 0, s>>>(g->dev.counts, host_counts, n);
}

int gfs_grep_run(gfs_grep* g, int n_ctas, float* kernel_ms) { return grep_run(g, n_ctas, kernel_ms, 0); }

int gfs_grep_run_direct(gfs_grep* g, int n_ctas, float* kernel_ms) { return grep_run(g, n_ctas, kernel_ms, 1); }

/* `steps` back-to-back runs on the kernel stream without host round trips;
 * *total_ms: events around all of them; *scan_ms: mean duration of the scan
 * kernel alone (events bracketing each launch on the same stream). */
int gfs_grep_bench(gfs_grep* g, int n_ctas, int steps, float* total_ms, float* scan_ms) {
    if (!g || steps < 1) return -GFS_EINVAL;
    if (gfs__activate(g->ctx)) return -GFS_EIO;
    cudaStream_t s = (cudaStream_t)gfs_kernel_stream(g->ctx);
    GrepDev& d = g->dev;
    if (n_ctas <= 0) n_ctas = g->sms;
    gfs_state* S = (gfs_state*)gfs_device_state(g->ctx);
    const int n_tail = tail_finish(g);
    if (n_tail < 0) return n_tail;
    std::vector<cudaEvent_t> ev((size_t)steps * 2 + 2);
    for (auto& e : ev) cudaEventCreate(&e);
    cudaMemsetAsync(d.status, 0, 8, s);
    set_window(g, n_ctas);
    cudaEventRecord(ev[0], s);
    for (int i = 0; i < steps; i++) {
        cudaMemsetAsync(d.counts, 0, (size_t)g->n_words * g->n_files * 4, s);
        cudaMemsetAsync(d.long_flags, 0, (size_t)g->n_files * 4, s);
        cudaEventRecord(ev[2 + 2 * (size_t)i], s);
        if (g->smem) k_grep_scan<true, false, false><<<n_ctas, GR_THREADS, g->smem_bytes, s>>>(S, d);
        else k_grep_scan<false, false, false><<<n_ctas, GR_THREADS, g->smem_bytes, s>>>(S, d);
        cudaEventRecord(ev[3 + 2 * (size_t)i], s);
        k_grep_fixup<<<g->n_files, 32, 0, s>>>(S, d);
        if (n_tail > 0) k_grep_tail<<<g->n_files, 32, 0, s>>>(S, d);
    }
    cudaEventRecord(ev[1], s);
    cudaError_t e = cudaEventSynchronize(ev[1]);
    float tot = 0, sum = 0;
    cudaEventElapsedTime(&tot, ev[0], ev[1]);
    for (int i = 0; i < steps; i++) {
        float x = 0;
        cudaEventElapsedTime(&x, ev[2 + 2 * (size_t)i], ev[3 + 2 * (size_t)i]);
        sum += x;
    }
    for (auto& x : ev) cudaEventDestroy(x);
    if (total_ms) *total_ms = tot;
    if (scan_ms) *scan_ms = sum / (float)steps;
    if (e != cudaSuccess) return -GFS_EIO;
    uint32_t status[2] = {0, 0};
    cudaMemcpy(status, d.status, 8, cudaMemcpyDeviceToHost);
    g->last_status[0] = status[0];
    g->last_status[1] = status[1];
    return status[0] ? -GFS_EIO : 0;
}

/* Batched run: every file's dictionary counts and XXH64 in one persistent
 * launch (CTAs take whole files, longest first), captured as a CUDA graph
 * on first use and replayed after. */
int gfs_grep_batch(gfs_grep* g, int n_ctas, unsigned long long* host_xxh, float* kernel_ms) {
    if (!g) return -GFS_EINVAL;
    if (gfs__activate(g->ctx)) return -GFS_EIO;
    cudaStream_t s = (cudaStream_t)gfs_kernel_stream(g->ctx);
    GrepDev& d = g->dev;
    if (n_ctas <= 0) n_ctas = g->sms;
    if (!g->batch_graph || g->batch_ctas != n_ctas) {
        if (g->batch_graph) cudaGraphExecDestroy(g->batch_graph);
        g->batch_graph = nullptr;
        set_window(g, n_ctas);
        gfs_state* S = (gfs_state*)gfs_device_state(g->ctx);
        cudaGraph_t graph = nullptr;
        /* thread-local capture: the host workers' copies on their own
         * streams go on while this thread records */
        if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return -GFS_EIO;
        cudaMemsetAsync(d.counts, 0, (size_t)g->n_words * g->n_files * 4, s);
        cudaMemsetAsync(d.long_flags, 0, (size_t)g->n_files * 4, s);
        cudaMemsetAsync(d.status, 0, 8, s);
        cudaMemsetAsync(d.file_next, 0, 4, s);
        if (g->smem) k_grep_scan<true, true, false><<<n_ctas, GR_THREADS, g->smem_bytes, s>>>(S, d);
        else k_grep_scan<false, true, false><<<n_ctas, GR_THREADS, g->smem_bytes, s>>>(S, d);
        k_grep_fixup<<<g->n_files, 32, 0, s>>>(S, d);
        cudaError_t ce = cudaStreamEndCapture(s, &graph);
        if (ce != cudaSuccess || !graph) return -GFS_EIO;
        ce = cudaGraphInstantiate(&g->batch_graph, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) {
            g->batch_graph = nullptr;
            return -GFS_EIO;
        }
        g->batch_ctas = n_ctas;
    }
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
    cudaError_t le = cudaGraphLaunch(g->batch_graph, s);
    const int n_tail = tail_finish(g); /* on the host while the batch runs */
    if (n_tail > 0) k_grep_tail<<<g->n_files, 32, 0, s>>>((gfs_state*)gfs_device_state(g->ctx), d);
    cudaEventRecord(b, s);
    cudaError_t e = cudaStreamSynchronize(s); /* kernels first, then copies back */
    if (kernel_ms) cudaEventElapsedTime(kernel_ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (le != cudaSuccess || e != cudaSuccess) {
        fprintf(stderr, "gpufs_gb300: batched grep failed: %s\n", cudaGetErrorString(le != cudaSuccess ? le : e));
        return -GFS_EIO;
    }
    uint32_t status[2] = {0, 0};
    cudaMemcpy(status, d.status, 8, cudaMemcpyDeviceToHost);
    g->last_status[0] = status[0];
    g->last_status[1] = status[1];
    if (host_xxh) cudaMemcpy(host_xxh, d.xxh, (size_t)g->n_files * 8, cudaMemcpyDeviceToHost);
    if (status[0]) return -((status[0] & GFS_ERRB_TIMEOUT) ? GFS_ETIMEDOUT : GFS_EIO);
    return n_tail < 0 ? n_tail : 0;
}

int gfs_grep_counts(gfs_grep* g, uint32_t* host_counts) {
    if (!g) return -GFS_EINVAL;
    cudaStream_t s = (cudaStream_t)gfs_kernel_stream(g->ctx);
    const size_t bytes = (size_t)g->n_words * g->n_files * 4;
    if (counts_out_ok(g, bytes)) {
        counts_out(g, host_counts, bytes, s);
        return cudaStreamSynchronize(s) == cudaSuccess && cudaGetLastError() == cudaSuccess ? 0 : -GFS_EIO;
    }
    /* through the session's pinned buffer: DMA at link speed, then a host
     * copy (a pageable copy is staged by the driver and much slower).  Up to
     * 1 GiB goes in one DMA and is copied out by several host threads (a
     * count matrix of thousands of files is hundreds of MB); larger ones go
     * 16 MiB at a time. */
    if (bytes > ((size_t)16 << 20) && bytes <= ((size_t)1 << 30)) {
        uint8_t* big = (uint8_t*)gfs__host_bounce(g->ctx, bytes);
        if (big) {
            if (cudaMemcpyAsync(big, g->dev.counts, bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess)
                return -GFS_EIO;
            unsigned nt = std::thread::hardware_concurrency();
            nt = nt < 1u ? 1u : (nt > 16u ? 16u : nt);
            if ((size_t)nt > bytes / ((size_t)8 << 20)) nt = (unsigned)(bytes / ((size_t)8 << 20));
            if (nt < 1u) nt = 1u;
            const size_t per = (bytes / nt + 4095u) & ~(size_t)4095u;
            std::vector<std::thread> th;
            for (unsigned i = 1; i < nt; i++) {
                const size_t a = per * i, e = a + per < bytes ? a + per : bytes;
                if (a < e) th.emplace_back([=] { memcpy((uint8_t*)host_counts + a, big + a, e - a); });
            }
            memcpy(host_counts, big, per < bytes ? per : bytes);
            for (auto& x : th) x.join();
            return 0;
        }
    }
    const size_t piece = bytes < ((size_t)16 << 20) ? bytes : ((size_t)16 << 20);
    void* hb = gfs__host_bounce(g->ctx, piece);
    if (hb) {
        for (size_t off = 0; off < bytes; off += piece) {
            const size_t n = bytes - off < piece ? bytes - off : piece;
            if (cudaMemcpyAsync(hb, (const uint8_t*)g->dev.counts + off, n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess)
                return -GFS_EIO;
            memcpy((uint8_t*)host_counts + off, hb, n);
        }
        return 0;
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) return -GFS_EIO;
    return cudaMemcpy(host_counts, g->dev.counts, bytes, cudaMemcpyDeviceToHost) == cudaSuccess ? 0 : -GFS_EIO;
}

int gfs_grep_info(gfs_grep* g, long long* out, int n) {
    long long v[10] = {g->n_words, g->n_files, (long long)g->m, g->smem ? 1 : 0, (long long)g->smem_bytes,
                       (long long)g->dev.total_chunks, (long long)g->last_status[0], (long long)g->last_status[1],
                       g->build_us, g->open_us};
    int k = n < 10 ? n : 10;
    for (int i = 0; i < k; i++) out[i] = v[i];
    return k;
}

void* gfs_grep_device_counts(gfs_grep* g) { return g ? (void*)g->dev.counts : nullptr; }

int gfs_grep_close(gfs_grep* g) {
    if (!g) return 0;
    int rc = 0;
    if (g->dmem && g->dev.fds) {
        gfs__activate(g->ctx);
        cudaStream_t s = (cudaStream_t)gfs_kernel_stream(g->ctx);
        int* rcs = (int*)gfs__dev_alloc(g->ctx, (size_t)g->n_files * 4, s);
        int* h = (int*)gfs__host_bounce(g->ctx, (size_t)g->n_files * 4);
        if (rcs && h) {
            k_close_files<<<g->n_files, 128, 0, s>>>(g->dev.fds, g->n_files, rcs);
            cudaMemcpyAsync(h, rcs, (size_t)g->n_files * 4, cudaMemcpyDeviceToHost, s);
            cudaStreamSynchronize(s);
            for (int i = 0; i < g->n_files; i++)
                if (h[i] < 0 && !rc) rc = h[i];
        }
        gfs__dev_free(g->ctx, rcs, s);
    }
    if (g->batch_graph) cudaGraphExecDestroy(g->batch_graph);
    gfs__dev_free(g->ctx, g->dmem, (cudaStream_t)gfs_kernel_stream(g->ctx));
    if (g->tail) cudaFreeHost(g->tail);
    delete g;
    return rc;
}

/* ---------------- served loop: host side ---------------- */
struct gfs_server {
    gfs_ctx* ctx = nullptr;
    gfs_grep* dict = nullptr; /* dictionary table (and no corpus) */
    int n_files = 0, n_out = 0;
    uint8_t* dmem = nullptr;  /* fds, sizes, out fds, names, head */
    int* fds = nullptr;
    uint64_t* sizes = nullptr;
    int* out_fds = nullptr;
    uint32_t* head = nullptr;
    SvPart* parts = nullptr;  /* part queue of split greps */
    unsigned long long last_hist[SV_HIST] = {}; /* the last run's service-time histogram */
    SvReq* ring_h = nullptr;  /* mapped */
    SvReq* ring_d = nullptr;
    uint32_t ring_n = 0;
    uint32_t* stop_h = nullptr; /* mapped */
    uint32_t* stop_d = nullptr;
    int sms = 0;
    std::vector<uint64_t> host_sizes;
};

/* part queue of a run: slot i free for position i, head = tail = 0 */
static __global__ void k_sv_reset(SvPart* parts, uint32_t* qht) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < SV_QCAP) parts[i].seq = i;
    if (i < 2u) qht[i] = 0u;
}

static uint64_t now_ns() {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec;
}

int gfs_serve_open(gfs_ctx* ctx, const char* dict_path, const char* const* paths, int n_files,
                   const char* const* out_paths, int n_out, gfs_server** out) {
    *out = nullptr;
    if (n_files < 1 || n_out < 0 || !dict_path) return -GFS_EINVAL;
    for (int i = 0; i < n_files; i++)
        if (!paths[i] || strlen(paths[i]) >= GFS_NAME_MAX) return -GFS_EINVAL;
    for (int i = 0; i < n_out; i++)
        if (!out_paths[i] || strlen(out_paths[i]) >= GFS_NAME_MAX) return -GFS_EINVAL;
    gfs_server* sv = new gfs_server();
    sv->ctx = ctx;
    sv->n_files = n_files;
    sv->n_out = n_out;
    /* the dictionary: a grep plan over no corpus file but the dictionary itself */
    const char* none[1] = {dict_path};
    int rc = gfs_grep_open(ctx, dict_path, none, 1, &sv->dict);
    if (rc < 0) { delete sv; return rc; }
    if (gfs__activate(ctx)) { gfs_serve_close(sv); return -GFS_EIO; }
    cudaStream_t s = (cudaStream_t)gfs_kernel_stream(ctx);
    const size_t n_all = (size_t)n_files + (size_t)n_out;
    size_t o_fds = 0, o_sz = align_up(o_fds + (size_t)n_files * 4, 256), o_ofd = align_up(o_sz + (size_t)n_files * 8, 256),
           o_osz = align_up(o_ofd + (size_t)n_out * 4 + 4, 256), o_head = align_up(o_osz + (size_t)n_out * 8 + 8, 256),
           o_parts = align_up(o_head + 64, 256), o_names = align_up(o_parts + (size_t)SV_QCAP * sizeof(SvPart), 256),
           total = align_up(o_names + n_all * GFS_NAME_MAX, 256);
    if (cudaMalloc(&sv->dmem, total) != cudaSuccess) { gfs_serve_close(sv); return -GFS_ENOMEM; }
    cudaMemset(sv->dmem, 0, total);
    sv->fds = (int*)(sv->dmem + o_fds);
    sv->sizes = (uint64_t*)(sv->dmem + o_sz);
    sv->out_fds = (int*)(sv->dmem + o_ofd);
    sv->head = (uint32_t*)(sv->dmem + o_head); /* ticket counter, then the part queue's head and tail */
    sv->parts = (SvPart*)(sv->dmem + o_parts);
    {
        std::vector<char> names(n_all * GFS_NAME_MAX, 0);
        for (int i = 0; i < n_files; i++) memcpy(&names[(size_t)i * GFS_NAME_MAX], paths[i], strlen(paths[i]));
        for (int i = 0; i < n_out; i++)
            memcpy(&names[((size_t)n_files + (size_t)i) * GFS_NAME_MAX], out_paths[i], strlen(out_paths[i]));
        cudaMemcpy(sv->dmem + o_names, names.data(), names.size(), cudaMemcpyHostToDevice);
    }
    /* every file opened once, for the server's life (the open-file table
     * stays on the device across requests) */
    k_open_files<<<n_files, 128, 0, s>>>((const char*)(sv->dmem + o_names), n_files, sv->fds, sv->sizes);
    if (n_out)
        k_open_files<<<n_out, 128, 0, s>>>((const char*)(sv->dmem + o_names) + (size_t)n_files * GFS_NAME_MAX, n_out,
                                           sv->out_fds, (uint64_t*)(sv->dmem + o_osz), O_GWRONCE);
    if (cudaStreamSynchronize(s) != cudaSuccess) { gfs_serve_close(sv); return -GFS_EIO; }
    std::vector<int> h((size_t)n_files + (size_t)n_out);
    cudaMemcpy(h.data(), sv->fds, (size_t)n_files * 4, cudaMemcpyDeviceToHost);
    if (n_out) cudaMemcpy(h.data() + n_files, sv->out_fds, (size_t)n_out * 4, cudaMemcpyDeviceToHost);
    sv->host_sizes.resize((size_t)n_files);
    cudaMemcpy(sv->host_sizes.data(), sv->sizes, (size_t)n_files * 8, cudaMemcpyDeviceToHost);
    for (int x : h)
        if (x < 0) { gfs_serve_close(sv); return x; }
    sv->ring_n = 1u << 16;
    if (cudaHostAlloc((void**)&sv->ring_h, (size_t)sv->ring_n * sizeof(SvReq), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&sv->ring_d, sv->ring_h, 0) != cudaSuccess ||
        cudaHostAlloc((void**)&sv->stop_h, 64, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&sv->stop_d, sv->stop_h, 0) != cudaSuccess) {
        gfs_serve_close(sv);
        return -GFS_ENOMEM;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sv->sms, cudaDevAttrMultiProcessorCount, dev);
    *out = sv;
    return 0;
}

/* Open-loop run: request k is published at (or after) its arrival time,
 * once the pages of the requests in flight leave room for it under
 * inflight_pages (memory-gated admission); latencies are completion minus
 * arrival, host clock.  warps_per_sm: serving warps per SM (multiple of 8). */
/* as many blocks as are resident at once: a queued block of this persistent
 * kernel would only start when others leave */
/* shared memory a served block stages the dictionary's tags and
 * displacements in (0 when they do not fit: the grep path then reads them
 * from global memory); the kernel attribute is raised to match */
static uint32_t serve_tbl_smem(gfs_server* sv) {
    const GrepDev& G = sv->dict->dev;
    const uint32_t bytes = grep_tag_smem(G.m) + grep_disp_smem(G.r);
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, k_serve) != cudaSuccess) return 0;
    if ((size_t)bytes + a.sharedSizeBytes > (size_t)optin) return 0;
    if (cudaFuncSetAttribute(k_serve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return bytes;
}

int gfs_serve_warps_per_sm(gfs_server* sv, int warps_per_sm) {
    if (!sv) return -GFS_EINVAL;
    if (gfs__activate(sv->ctx)) return -GFS_EIO;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_serve, SV_WARPS * 32, serve_tbl_smem(sv)) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 0; /* unknown: no cap */
    }
    int bps = warps_per_sm / SV_WARPS;
    if (bps < 1) bps = 1;
    if (per_sm > 0 && bps > per_sm) bps = per_sm;
    return bps * SV_WARPS;
}

int gfs_serve_run(gfs_server* sv, const gfs_serve_req* reqs, int n, gfs_serve_res* res, uint64_t inflight_pages,
                  int warps_per_sm) {
    if (!sv || n < 0 || (n && (!reqs || !res))) return -GFS_EINVAL;
    if (gfs__activate(sv->ctx)) return -GFS_EIO;
    if (warps_per_sm < SV_WARPS) warps_per_sm = SV_WARPS;
    cudaStream_t s = (cudaStream_t)gfs_kernel_stream(sv->ctx);
    SvComp* comp_h = nullptr;
    SvComp* comp_d = nullptr;
    if (cudaHostAlloc((void**)&comp_h, (size_t)(n ? n : 1) * sizeof(SvComp), cudaHostAllocMapped) != cudaSuccess)
        return -GFS_ENOMEM;
    cudaHostGetDevicePointer((void**)&comp_d, comp_h, 0);
    memset(comp_h, 0, (size_t)(n ? n : 1) * sizeof(SvComp));
    for (uint32_t i = 0; i < sv->ring_n; i++) __atomic_store_n(&sv->ring_h[i].seq, i, __ATOMIC_RELAXED);
    __atomic_store_n(sv->stop_h, 0u, __ATOMIC_RELEASE);
    cudaMemsetAsync(sv->head, 0, 4, s);
    /* an accumulator per request id (split greps, service start times), the
     * part queue reset, the service-time histogram after the accumulators */
    const size_t acc_bytes = ((size_t)(n ? n : 1) * sizeof(SvAcc) + 255u) & ~(size_t)255u;
    SvAcc* acc = (SvAcc*)gfs__dev_alloc(sv->ctx, acc_bytes + SV_HIST * 8, s);
    if (!acc) { cudaFreeHost(comp_h); return -GFS_ENOMEM; }
    unsigned long long* hist = (unsigned long long*)((uint8_t*)acc + acc_bytes);
    cudaMemsetAsync(acc, 0, acc_bytes + SV_HIST * 8, s);
    k_sv_reset<<<(SV_QCAP + 255u) / 256u, 256, 0, s>>>(sv->parts, sv->head + 1);
    ServeDev D{};
    D.G = sv->dict->dev;
    D.ring = sv->ring_d;
    D.ring_mask = sv->ring_n - 1u;
    D.head = sv->head;
    D.comp = comp_d;
    D.fds = sv->fds;
    D.sizes = sv->sizes;
    D.out_fds = sv->out_fds;
    D.n_files = sv->n_files;
    D.n_out = sv->n_out;
    D.stop = sv->stop_d;
    D.acc = acc;
    D.parts = sv->parts;
    D.q_head = sv->head + 1;
    D.q_tail = sv->head + 2;
    D.tbl_smem = serve_tbl_smem(sv);
    D.hist = hist;
    const uint32_t page = gfs_page_size(sv->ctx);
    const int blocks = sv->sms * (gfs_serve_warps_per_sm(sv, warps_per_sm) / SV_WARPS);
    k_serve<<<blocks, SV_WARPS * 32, D.tbl_smem, s>>>((gfs_state*)gfs_device_state(sv->ctx), D);
    if (cudaGetLastError() != cudaSuccess) {
        gfs__dev_free(sv->ctx, acc, s);
        cudaFreeHost(comp_h);
        return -GFS_EIO;
    }
    std::vector<uint32_t> cost((size_t)n);
    for (int k = 0; k < n; k++) cost[(size_t)k] = (uint32_t)((reqs[k].length + page - 1) / page) + 1u;
    std::atomic<uint64_t> inflight{0};
    std::atomic<int> submitted{0}, completed{0};
    std::atomic<int> quit{0};
    const uint64_t t0 = now_ns();
    /* completions: scanned in submission order from the oldest open one */
    std::thread poller([&] {
        std::vector<char> seen((size_t)n, 0);
        int lo = 0;
        while (completed.load() < n && !quit.load()) {
            const int hi = submitted.load(std::memory_order_acquire);
            bool any = false;
            for (int k = lo; k < hi; k++) {
                if (seen[(size_t)k]) continue;
                if (__atomic_load_n(&comp_h[k].done, __ATOMIC_ACQUIRE)) {
                    res[k].complete_ns = now_ns() - t0;
                    res[k].result = comp_h[k].result;
                    res[k].status = comp_h[k].status;
                    seen[(size_t)k] = 1;
                    inflight.fetch_sub(cost[(size_t)k]);
                    completed.fetch_add(1);
                    any = true;
                }
            }
            while (lo < hi && seen[(size_t)lo]) lo++;
            if (!any) sched_yield();
        }
    });
    const uint64_t limit_ns = 4ull * gfs__timeout_ns(sv->ctx) + 1000000000ull;
    int rc = 0;
    for (int k = 0; k < n && !rc; k++) {
        const uint64_t due = reqs[k].arrival_ns;
        while (now_ns() - t0 < due) {
        }
        /* memory-gated admission */
        while (inflight.load() + cost[(size_t)k] > inflight_pages && inflight.load() > 0) {
            if (now_ns() - t0 > due + limit_ns) { rc = -GFS_ETIMEDOUT; break; }
        }
        if (rc) break;
        SvReq* slot = &sv->ring_h[(uint32_t)k & (sv->ring_n - 1u)];
        while (__atomic_load_n(&slot->seq, __ATOMIC_ACQUIRE) != (uint32_t)k) {
            if (now_ns() - t0 > due + limit_ns) { rc = -GFS_ETIMEDOUT; break; }
        }
        if (rc) break;
        slot->op = reqs[k].op;
        slot->file = reqs[k].file;
        slot->id = (uint32_t)k;
        slot->offset = reqs[k].offset;
        slot->length = reqs[k].length;
        res[k].submit_ns = now_ns() - t0;
        inflight.fetch_add(cost[(size_t)k]);
        __atomic_store_n(&slot->seq, (uint32_t)k + 1u, __ATOMIC_RELEASE);
        submitted.store(k + 1, std::memory_order_release);
    }
    const uint64_t wait_from = now_ns();
    while (!rc && completed.load() < n) {
        if (now_ns() - wait_from > limit_ns) { rc = -GFS_ETIMEDOUT; break; }
        sched_yield();
    }
    quit.store(1);
    __atomic_store_n(sv->stop_h, 1u, __ATOMIC_RELEASE);
    cudaError_t e = cudaStreamSynchronize(s);
    poller.join();
    if (e == cudaSuccess) e = cudaMemcpy(sv->last_hist, hist, sizeof sv->last_hist, cudaMemcpyDeviceToHost);
    gfs__dev_free(sv->ctx, acc, s);
    cudaFreeHost(comp_h);
    if (e != cudaSuccess) return -GFS_EIO;
    return rc;
}

int gfs_serve_service_hist(gfs_server* sv, unsigned long long* out, int n) {
    if (!sv || n < 0 || (n && !out)) return -GFS_EINVAL;
    const int k = n < SV_HIST ? n : SV_HIST;
    for (int i = 0; i < k; i++) out[i] = sv->last_hist[i];
    return SV_HIST;
}

int gfs_serve_close(gfs_server* sv) {
    if (!sv) return 0;
    int rc = 0;
    if (sv->dmem && sv->fds) {
        gfs__activate(sv->ctx);
        cudaStream_t s = (cudaStream_t)gfs_kernel_stream(sv->ctx);
        int* rcs = nullptr;
        const int n_all = sv->n_files + sv->n_out;
        if (n_all && cudaMalloc(&rcs, (size_t)n_all * 4) == cudaSuccess) {
            k_close_files<<<sv->n_files, 128, 0, s>>>(sv->fds, sv->n_files, rcs);
            if (sv->n_out) k_close_files<<<sv->n_out, 128, 0, s>>>(sv->out_fds, sv->n_out, rcs + sv->n_files);
            cudaStreamSynchronize(s);
            std::vector<int> h((size_t)n_all);
            cudaMemcpy(h.data(), rcs, h.size() * 4, cudaMemcpyDeviceToHost);
            for (int x : h)
                if (x < 0 && !rc) rc = x;
            cudaFree(rcs);
        }
    }
    if (sv->ring_h) cudaFreeHost(sv->ring_h);
    if (sv->stop_h) cudaFreeHost(sv->stop_h);
    cudaFree(sv->dmem);
    if (sv->dict) gfs_grep_close(sv->dict);
    delete sv;
    return rc;
}

int gfs_grep_text(gfs_ctx* ctx, const char* dict_path, const char* const* paths, int n_files, uint32_t* host_counts,
                  int n_ctas) {
    gfs_grep* g = nullptr;
    int rc = gfs_grep_open(ctx, dict_path, paths, n_files, &g);
    if (rc) return rc;
    /* one pass, read straight from the files' mappings; the counts come
     * back with the run's own synchronisation where the device may write
     * the caller's memory */
    const bool merged = counts_out_ok(g, (size_t)g->n_words * g->n_files * 4);
    rc = grep_run(g, n_ctas, nullptr, 1, merged ? host_counts : nullptr);
    if (!rc && !merged) rc = gfs_grep_counts(g, host_counts);
    int c = gfs_grep_close(g);
    return rc ? rc : c;
}

} /* extern "C" */

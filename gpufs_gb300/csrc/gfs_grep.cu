/*
 * grep_text over the GPU file system: whole-word occurrence counts of every
 * dictionary record in every corpus file, read through the HBM buffer cache.
 *
 * Reference: samples/grep_text/grep_text_gpu.cu:193-387 (kernel grep_text),
 * :139-160 (match_string), :79 (alpha).  The reference gives each thread one
 * dictionary word and rescans every 16 KiB corpus chunk for it -- O(words x
 * corpus bytes).  Here the corpus is read once:
 *
 *   - one persistent 1024-thread CTA per SM owns a contiguous run of 16 KiB
 *     chunks of the concatenated corpus; warp 0 pins the run's pages in the
 *     buffer cache 32 at a time (one lane per page, host reads in parallel
 *     on a miss) and thread 0 streams chunks from the page frames into a
 *     4-stage shared-memory ring with 1D TMA bulk copies (cp.async.bulk,
 *     mbarrier completion, bounded waits);
 *   - each warp classifies a 512-byte segment with SWAR byte arithmetic
 *     (16 bytes per lane), finds token starts/ends from the alpha bitmasks
 *     and a shuffle across lanes, and compacts the tokens into a per-warp
 *     list so every lane works on one token;
 *   - a token is hashed from its zero-padded bytes and looked up in a
 *     bucketised cuckoo table (2 choices x 4 slots, 12-bit tags) held in
 *     shared memory; a tag hit is verified against the 32-byte record (L2),
 *     and the slot's 20-bit counter in shared memory is incremented;
 *   - counters are flushed to counts[word][file] with global atomics when
 *     the CTA moves to another file (or a counter reaches 2^19).
 *
 * Exactness: a token counts for record w iff it equals w (match_string
 * semantics; empty records never match, duplicate records all count).  The
 * reference's chunk walk additionally cuts an alpha run when the 32 bytes
 * after a 16384-byte window are all letters (grep_text_gpu.cu:302-318); runs
 * of >= 33 letters are flagged per file and k_grep_fixup restates that walk
 * for flagged files only, so counts equal the reference on any input.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <errno.h>
#include <fcntl.h>
#include <unistd.h>
#include <sys/stat.h>

#include <algorithm>
#include <string>
#include <unordered_map>
#include <vector>

#include "gfs_device.cuh"
#include "gfs_block.cuh"
#include "gfs_grep_common.h"
#include "gfs_runtime.h"
#include "gpufs_gb300.h"

#define GR_CH 16384
#define GR_STAGES 4
#define GR_THREADS 1024
#define GR_WARPS 32
#define GR_SEG 512
#define GR_LIST 256
#define GR_WIN 32 /* pages pinned per window, including look-behind/ahead */

extern __device__ gfs_state* g_gfs;

struct GrepDev {
    int n_files;
    int n_words;
    const int* fds;
    const uint64_t* sizes;
    const uint64_t* chunk_prefix; /* n_files + 1 */
    uint64_t total_chunks;
    uint32_t nb;                  /* buckets */
    const uint32_t* table;        /* nb * 4 slot words: tag << 20 */
    const uint4* recs;            /* nb * 4 records of 32 bytes */
    const uint32_t* slot_word;    /* first record of each slot, ~0 if empty */
    const int32_t* next_dup;      /* next record with the same word, -1 */
    uint32_t* counts;             /* n_words x n_files */
    uint32_t* long_flags;         /* per file: a run of >= 33 letters was seen */
    uint32_t* status;             /* [0] error bits, [1] first failure: site << 16 | errno */
    uint32_t win_data;            /* data pages per window (window = data + look-behind/ahead) */
};

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
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok) : "r"(smem_u32(b)), "r"(parity) : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

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
__device__ __forceinline__ bool is_alpha(uint32_t c) {
    return (c - 65u < 26u) || (c - 97u < 26u) || c == 95u;
}

/* zero-padded key words of `len` (1..32) bytes starting at byte `st` of an
 * smem buffer that is readable 4 bytes past st+len */
__device__ __forceinline__ void key_from_smem(const uint8_t* base, uint32_t st, int len, uint32_t k[8]) {
    const uint32_t* w = (const uint32_t*)(base + (st & ~3u));
    const uint32_t sh = (st & 3u) * 8u;
    const int nw = (int)(((st & 3u) + (uint32_t)len + 3u) >> 2);
    uint32_t x[9];
#pragma unroll
    for (int i = 0; i < 9; i++) x[i] = (i < nw) ? w[i] : 0u;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        uint32_t v = __funnelshift_r(x[i], x[i + 1], sh);
        int valid = len - 4 * i;
        uint32_t m = valid >= 4 ? 0xFFFFFFFFu : (valid <= 0 ? 0u : ((1u << (8 * valid)) - 1u));
        k[i] = v & m;
    }
}

struct Ctx {
    gfs_state* S;
    GrepDev P;
    uint32_t lp, pmask;
};

/* shared state of a CTA */
struct Shared {
    uint64_t mbar[GR_STAGES];
    int win_frames[GR_WIN];
    uint32_t win_lb;      /* first pinned page */
    int win_n;            /* pinned pages */
    int err;
    uint32_t prev_alpha[2];
};

__device__ __forceinline__ uint32_t gbyte(const Ctx& C, const Shared& sh, uint64_t fsize, uint64_t q) {
    if (q >= fsize) return 0u;
    uint32_t pg = (uint32_t)(q >> C.lp);
    int i = (int)(pg - sh.win_lb);
    if (i < 0 || i >= sh.win_n) return 0u; /* not pinned: cannot happen within 33 bytes of a window */
    const uint8_t* p = C.S->pool + ((size_t)sh.win_frames[i] << C.lp) + (q & C.pmask);
    return (uint32_t)__ldcg(p);
}

__device__ __forceinline__ void flush_slot(const GrepDev& P, uint32_t slot, uint32_t n, int f) {
    uint32_t w = P.slot_word[slot];
    while (w != 0xFFFFFFFFu && (int)w < P.n_words) {
        atomicAdd(&P.counts[(size_t)w * P.n_files + f], n);
        int32_t d = P.next_dup[w];
        w = d < 0 ? 0xFFFFFFFFu : (uint32_t)d;
    }
}

/* Look a key up; on a verified match count it (smem counter or global). */
template <bool SMEM>
__device__ __forceinline__ void count_key(const GrepDev& P, uint32_t* tbl, const uint32_t k[8], int len, int f) {
    uint64_t h = grep_hash(k, len);
    uint32_t tag = grep_tag(h);
    uint32_t bs[2] = {grep_b1(h, P.nb), grep_b2(h, P.nb)};
#pragma unroll
    for (int r = 0; r < 2; r++) {
        uint4 q = SMEM ? *(const uint4*)(tbl + 4u * bs[r]) : __ldg((const uint4*)(P.table + 4u * bs[r]));
        uint32_t s4[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int i = 0; i < 4; i++) {
            if ((s4[i] >> GREP_TAG_SHIFT) != tag) continue;
            uint32_t slot = 4u * bs[r] + (uint32_t)i;
            uint4 a = __ldg(P.recs + 2u * slot), b = __ldg(P.recs + 2u * slot + 1u);
            if (a.x == k[0] && a.y == k[1] && a.z == k[2] && a.w == k[3] && b.x == k[4] && b.y == k[5] &&
                b.z == k[6] && b.w == k[7]) {
                if (SMEM) {
                    uint32_t old = atomicAdd(&tbl[slot], 1u);
                    if ((old & GREP_CNT_MASK) == 0x7FFFFu) { /* keep the 20-bit counter from overflowing */
                        atomicSub(&tbl[slot], 0x80000u);
                        flush_slot(P, slot, 0x80000u, f);
                    }
                } else {
                    flush_slot(P, slot, 1u, f);
                }
                return;
            }
        }
    }
}

/* Pin the window's pages (warp 0; one lane per page).  Returns 0, -GFS_ENOMEM
 * when the pool could not hold the whole window (nothing is left pinned;
 * the caller shrinks the window), or another -err. */
__device__ int pin_window(const Ctx& C, Shared& sh, int fd, uint64_t fsize, uint32_t lb, int n) {
    const int lane = threadIdx.x & 31;
    int r = 0;
    if (lane < n) {
        PinFile pf = pin_file(C.S, fd);
        bool fresh;
        r = pin_page(C.S, pf, lb + (uint32_t)lane, GFS_PIN_READ | (n > 1 ? GFS_PIN_NOALLOC : 0), &fresh);
        if (r >= 0 && fresh) { /* beyond the host file: cannot happen below fsize */
            publish_valid(C.S, (uint32_t)r);
        }
        sh.win_frames[lane] = r;
    }
    unsigned bad = __ballot_sync(0xFFFFFFFFu, lane < n && r < 0 && r != -GFS_ENOMEM);
    unsigned nomem = __ballot_sync(0xFFFFFFFFu, lane < n && r == -GFS_ENOMEM);
    if (bad || nomem) {
        if (lane < n && r >= 0) unpin(C.S, (uint32_t)r);
        return bad ? __shfl_sync(0xFFFFFFFFu, r, __ffs(bad) - 1) : -GFS_ENOMEM;
    }
    return 0;
}

__device__ void unpin_window(const Ctx& C, Shared& sh) {
    const int lane = threadIdx.x & 31;
    if (lane < sh.win_n) unpin(C.S, (uint32_t)sh.win_frames[lane]);
}

/* Process one staged chunk.  base: the stage buffer (chunk byte 0),
 * clen: valid bytes, cpos: file offset of the chunk. */
template <bool SMEM>
__device__ __forceinline__ void scan_chunk(const Ctx& C, Shared& sh, uint32_t* tbl, const uint8_t* base, uint32_t clen,
                                           uint32_t avail, uint64_t cpos, uint64_t fsize, int f, uint16_t* slist,
                                           uint16_t* elist, uint8_t* wscratch, int parity) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t seg0 = (uint32_t)warp * GR_SEG;
    const bool last_in_file = cpos + clen >= fsize;
    if (seg0 < clen) {
        const uint32_t off = seg0 + 16u * (uint32_t)lane;
        uint4 v = *(const uint4*)(base + off);
        uint32_t a = alpha16(v);
        if (off >= clen) a = 0u;
        else if (clen - off < 16u) a &= (1u << (clen - off)) - 1u;
        /* previous byte's class */
        uint32_t pb = __shfl_up_sync(0xFFFFFFFFu, a >> 15, 1);
        if (lane == 0) pb = (seg0 == 0) ? sh.prev_alpha[parity] : (uint32_t)is_alpha(base[seg0 - 1]);
        /* next byte's class; past the chunk end a token may continue (it is
         * then left open and its end found by a scan), past the file end not */
        uint32_t nxt = __shfl_down_sync(0xFFFFFFFFu, a & 1u, 1);
        if (lane == 31) nxt = seg0 + GR_SEG < clen ? (uint32_t)is_alpha(base[seg0 + GR_SEG]) : 0u;
        uint32_t na = (a >> 1) | (nxt << 15);
        if (off < clen && clen - off <= 16u) {
            const uint32_t j = clen - off - 1u;
            na = (na & ~(1u << j)) | ((last_in_file ? 0u : 1u) << j);
        }
        const uint32_t starts = a & ~((a << 1) | pb) & 0xFFFFu;
        const uint32_t ends = a & ~na;
        const uint32_t ns = (uint32_t)__popc(starts), ne = (uint32_t)__popc(ends);
        uint32_t packed = ns | (ne << 16), incl = packed;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= d) incl += t;
        }
        const uint32_t excl = incl - packed;
        const uint32_t tot = __shfl_sync(0xFFFFFFFFu, incl, 31);
        const uint32_t n_s = tot & 0xFFFFu, n_e = tot >> 16;
        uint32_t js = excl & 0xFFFFu, je = excl >> 16;
        for (uint32_t m = starts; m; m &= m - 1u) slist[js++] = (uint16_t)(off + (uint32_t)(__ffs(m) - 1));
        for (uint32_t m = ends; m; m &= m - 1u) elist[je++] = (uint16_t)(off + (uint32_t)(__ffs(m) - 1));
        /* does the segment begin inside a token started earlier? */
        const uint32_t carry = __shfl_sync(0xFFFFFFFFu, (a & 1u) & pb, 0);
        __syncwarp();
        for (uint32_t t = (uint32_t)lane; t < n_s; t += 32u) {
            const uint32_t st = slist[t];
            const uint32_t ei = t + carry;
            int len;
            bool in_stage;
            if (ei < n_e) {
                len = (int)elist[ei] - (int)st + 1;
                in_stage = true;
            } else {
                /* open at the segment end: scan forward through the staged
                 * bytes (chunk + look-ahead); past `avail` lies end of file */
                uint32_t p = st + 1u;
                bool open = true;
                while (open && p - st <= 32u) {
                    uint32_t c = p < avail ? base[p] : (cpos + p >= fsize ? 0u : gbyte(C, sh, fsize, cpos + p));
                    if (!is_alpha(c)) open = false;
                    else p++;
                }
                len = (int)(p - st);
                in_stage = p <= avail; /* always, given 64 bytes of look-ahead */
                if (open) len = 33;
            }
            if (len > 32) {
                if (len >= 33) atomicOr(&C.P.long_flags[f], 1u);
                continue;
            }
            uint32_t k[8];
            if (in_stage) {
                key_from_smem(base, st, len, k);
            } else {
                /* crosses the chunk end: gather into this lane's scratch */
                uint8_t* s = wscratch; /* one token per chunk crosses its end */
                for (int i = 0; i < 40; i++) s[i] = 0;
                for (int i = 0; i < len; i++) {
                    uint32_t p = st + (uint32_t)i;
                    s[i] = (uint8_t)(p < clen ? base[p] : gbyte(C, sh, fsize, cpos + p));
                }
                key_from_smem(s, 0, len, k);
            }
            count_key<SMEM>(C.P, tbl, k, len, f);
        }
    }
    /* the last valid byte's class is the next chunk's look-behind */
    if (threadIdx.x == 0) {
        uint32_t lb = clen ? (uint32_t)is_alpha(base[clen - 1]) : sh.prev_alpha[parity];
        sh.prev_alpha[parity ^ 1] = lb;
    }
}

template <bool SMEM>
__device__ void flush_counts(const Ctx& C, uint32_t* tbl, int f) {
    if (!SMEM) return;
    const uint32_t nslots = 4u * C.P.nb;
    for (uint32_t i = threadIdx.x; i < nslots; i += blockDim.x) {
        uint32_t v = tbl[i];
        uint32_t n = v & GREP_CNT_MASK;
        if (n) {
            tbl[i] = v & ~GREP_CNT_MASK;
            flush_slot(C.P, i, n, f);
        }
    }
}

} // namespace

/* One persistent CTA per SM; see the file comment. */
template <bool SMEM>
__global__ void __launch_bounds__(GR_THREADS, 1) k_grep_scan(gfs_state* S, GrepDev P) {
    extern __shared__ __align__(128) uint8_t dsm[];
    __shared__ Shared sh;
    Ctx C;
    C.S = S;
    C.P = P;
    C.lp = S->log_page;
    C.pmask = S->page_size - 1u;
    const uint32_t tbl_bytes = SMEM ? 16u * P.nb : 0u;
    uint32_t* tbl = SMEM ? (uint32_t*)dsm : (uint32_t*)P.table;
    uint8_t* stages = dsm + ((tbl_bytes + 127u) & ~127u);
    const uint32_t stage_bytes = GR_CH + 96u; /* chunk + 64 look-ahead + read slack */
    uint16_t* lists = (uint16_t*)(stages + GR_STAGES * stage_bytes);
    uint8_t* scratch = (uint8_t*)(lists + GR_WARPS * 2 * GR_LIST);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint16_t* slist = lists + warp * 2 * GR_LIST;
    uint16_t* elist = slist + GR_LIST;
    uint8_t* wscratch = scratch + warp * 48;

    if (SMEM)
        for (uint32_t i = threadIdx.x; i < P.nb; i += blockDim.x) ((uint4*)tbl)[i] = __ldg((const uint4*)P.table + i);
    if (threadIdx.x == 0) {
        for (int s = 0; s < GR_STAGES; s++) mbar_init(&sh.mbar[s], 1u);
        fence_mbar_init();
        sh.err = 0;
        sh.prev_alpha[0] = sh.prev_alpha[1] = 0u;
    }
    __syncthreads();

    const uint64_t total = P.total_chunks;
    const uint64_t c0 = total * blockIdx.x / gridDim.x, c1 = total * (blockIdx.x + 1) / gridDim.x;
    uint32_t gi = 0; /* chunks streamed by this CTA: stage = gi % STAGES, parity = (gi / STAGES) & 1 */
    int parity = 0;   /* prev_alpha double buffer */
    const uint32_t page = S->page_size;
    const uint32_t chunks_per_page = page >= GR_CH ? page / GR_CH : 1u;
    const uint32_t pages_per_chunk = page >= GR_CH ? 1u : GR_CH / page;
    __shared__ uint32_t s_wdp; /* data pages per window; halved when the pool is short */
    if (threadIdx.x == 0) {
        uint32_t w = P.win_data ? P.win_data : (GR_WIN - 2);
        if (w > GR_WIN - 2) w = GR_WIN - 2;
        w = w / pages_per_chunk * pages_per_chunk;
        s_wdp = w ? w : pages_per_chunk;
    }
    __syncthreads();

    uint64_t cur = c0;
    while (cur < c1 && !sh.err) {
        /* file of chunk `cur` */
        int lo = 0, hi = P.n_files - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (P.chunk_prefix[mid] <= cur) lo = mid; else hi = mid - 1;
        }
        const int f = lo;
        const uint64_t fend = P.chunk_prefix[f + 1] < c1 ? P.chunk_prefix[f + 1] : c1;
        const uint64_t fsize = P.sizes[f];
        const int fd = P.fds[f];
        const uint32_t fpages = (uint32_t)((fsize + page - 1) >> C.lp);
        uint64_t k = cur - P.chunk_prefix[f];  /* chunk index within the file */
        const uint64_t kend = fend - P.chunk_prefix[f];
        bool first_window = true;
        while (k < kend && !sh.err) {
            /* window: data pages from the page of chunk k */
            const uint32_t dp0 = (uint32_t)((k * GR_CH) >> C.lp);
            uint32_t dp1 = dp0 + s_wdp;
            const uint32_t need_end = (uint32_t)(((kend * GR_CH < fsize ? kend * GR_CH : fsize) + page - 1) >> C.lp);
            if (dp1 > need_end) dp1 = need_end;
            uint32_t lb = dp0;
            if (first_window && k * GR_CH > 0) lb = (uint32_t)((k * GR_CH - 1) >> C.lp);
            uint32_t ub = dp1 + 1u < fpages ? dp1 + 1u : fpages; /* look-ahead page */
            if (ub < dp1) ub = dp1;
            const uint64_t kw_end_pos = (uint64_t)dp1 << C.lp;
            uint64_t kw_end = (kw_end_pos + GR_CH - 1) / GR_CH;
            if (kw_end > kend) kw_end = kend;
            if (warp == 0) {
                if (lane == 0) {
                    sh.win_lb = lb;
                    sh.win_n = (int)(ub - lb);
                }
                __syncwarp();
                int e = pin_window(C, sh, fd, fsize, lb, (int)(ub - lb));
                if (lane == 0 && e) {
                    if (e == -GFS_ENOMEM && s_wdp > pages_per_chunk) {
                        s_wdp = (s_wdp / 2 + pages_per_chunk - 1) / pages_per_chunk * pages_per_chunk;
                        sh.err = 1; /* retry this window smaller */
                    } else {
                        sh.err = e;
                        atomicCAS(&P.status[1], 0u, (2u << 16) | (uint32_t)(-e));
                    }
                }
            }
            __syncthreads();
            if (sh.err == 1) {
                __syncthreads();
                if (threadIdx.x == 0) sh.err = 0;
                __syncthreads();
                continue;
            }
            if (sh.err) break;
            if (threadIdx.x == 0 && first_window) {
                sh.prev_alpha[parity] = k == 0 ? 0u : (uint32_t)is_alpha(gbyte(C, sh, fsize, k * GR_CH - 1));
            }
            first_window = false;
            /* stream chunks [k, kw_end) through the stage ring */
            const uint32_t n = (uint32_t)(kw_end - k);
            auto issue = [&](uint32_t i) {
                const uint64_t kk = k + i;
                const uint32_t g = gi + i;
                uint8_t* dst = stages + (g % GR_STAGES) * stage_bytes;
                uint64_t pos = kk * GR_CH;
                /* the chunk plus 64 bytes of look-ahead (tokens that start in the
                 * chunk end at most 33 bytes past it), rounded to 16 bytes */
                uint64_t cov = fsize - pos < (uint64_t)GR_CH + 64u ? fsize - pos : (uint64_t)GR_CH + 64u;
                uint32_t clen16 = ((uint32_t)cov + 15u) & ~15u;
                mbar_expect_tx(&sh.mbar[g % GR_STAGES], clen16);
                uint32_t done = 0;
                while (done < clen16) {
                    uint64_t q = pos + done;
                    uint32_t pg = (uint32_t)(q >> C.lp);
                    uint32_t in_pg = (uint32_t)(q & C.pmask);
                    uint32_t piece = page - in_pg;
                    if (piece > clen16 - done) piece = clen16 - done;
                    const uint8_t* src = S->pool + ((size_t)sh.win_frames[pg - sh.win_lb] << C.lp) + in_pg;
                    bulk_g2s(dst + done, src, piece, &sh.mbar[g % GR_STAGES]);
                    done += piece;
                }
            };
            if (threadIdx.x == 0) {
                fence_proxy_async();
                for (uint32_t i = 0; i < n && i < GR_STAGES - 1; i++) issue(i);
            }
            for (uint32_t i = 0; i < n; i++) {
                const uint32_t g = gi + i;
                if (threadIdx.x == 0 && i + GR_STAGES - 1 < n) {
                    fence_proxy_async();
                    issue(i + GR_STAGES - 1);
                }
                /* wait for chunk i (bounded) */
                {
                    uint32_t spins = 0;
                    while (!mbar_try_wait(&sh.mbar[g % GR_STAGES], (g / GR_STAGES) & 1u)) {
                        if (++spins > (1u << 26)) {
                            if (threadIdx.x == 0) {
                                sh.err = -GFS_ETIMEDOUT;
                                atomicOr(P.status, GFS_ERRB_TIMEOUT);
                                atomicCAS(&P.status[1], 0u, (1u << 16) | (uint32_t)(g & 0xFFFFu));
                            }
                            break;
                        }
                        if (spins > 64) __nanosleep(64);
                    }
                }
                const uint64_t kk = k + i;
                const uint64_t pos = kk * GR_CH;
                const uint32_t clen = (uint32_t)(fsize - pos < GR_CH ? fsize - pos : GR_CH);
                const uint32_t avail = (uint32_t)(fsize - pos < (uint64_t)GR_CH + 64u ? fsize - pos : (uint64_t)GR_CH + 64u);
                const uint8_t* base = stages + (g % GR_STAGES) * stage_bytes;
                scan_chunk<SMEM>(C, sh, tbl, base, clen, avail, pos, fsize, f, slist, elist, wscratch, parity);
                parity ^= 1;
                __syncthreads();
            }
            gi += n;
            if (warp == 0) unpin_window(C, sh);
            __syncthreads();
            k = kw_end;
        }
        flush_counts<SMEM>(C, tbl, f);
        __syncthreads();
        cur = fend;
    }
    if (threadIdx.x == 0 && sh.err) atomicOr(P.status, sh.err == -GFS_ETIMEDOUT ? GFS_ERRB_TIMEOUT : GFS_ERRB_IO);
    (void)chunks_per_page;
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
    count_key<false>(P, nullptr, k, len, f);
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

template __global__ void k_grep_scan<true>(gfs_state*, GrepDev);
template __global__ void k_grep_scan<false>(gfs_state*, GrepDev);

/* ------------------------------------------------------------------ */
/* host side: dictionary table, file opening, launch                   */
/* ------------------------------------------------------------------ */
static __global__ void k_open_files(const char* names, int n, int* fds, uint64_t* sizes) {
    int f = blockIdx.x;
    if (f >= n) return;
    gfs_state* S = g_gfs;
    int fd = gfsd::blk_open(S, names + (size_t)f * GFS_NAME_MAX, O_GRDONLY);
    if (threadIdx.x == 0) {
        fds[f] = fd;
        sizes[f] = fd >= 0 ? gfsd::ld_rlx64(&S->files[fd].size) : 0;
    }
}

static __global__ void k_close_files(const int* fds, int n, int* rcs) {
    int f = blockIdx.x;
    if (f >= n) return;
    int fd = fds[f];
    int r = fd >= 0 ? gfsd::blk_close(g_gfs, fd) : 0;
    if (threadIdx.x == 0) rcs[f] = r;
}

namespace {

struct HostTable {
    uint32_t nb = 0;
    std::vector<uint32_t> tbl;       /* nb*4 */
    std::vector<uint32_t> recs;      /* nb*4*8 */
    std::vector<uint32_t> slot_word; /* nb*4 */
    std::vector<int32_t> next_dup;   /* n_words */
};

void rec_key(const uint8_t* rec, uint32_t k[8], int* len) {
    int l = 0;
    while (l < 32 && rec[l]) l++;
    uint8_t b[32] = {0};
    memcpy(b, rec, (size_t)l);
    for (int i = 0; i < 8; i++)
        k[i] = (uint32_t)b[4 * i] | ((uint32_t)b[4 * i + 1] << 8) | ((uint32_t)b[4 * i + 2] << 16) |
               ((uint32_t)b[4 * i + 3] << 24);
    *len = l;
}

bool build_table(const uint8_t* dict, int n_words, HostTable& T) {
    std::unordered_map<std::string, int> first;
    std::vector<int> uniq;
    T.next_dup.assign((size_t)(n_words > 0 ? n_words : 1), -1);
    std::vector<int> last((size_t)(n_words > 0 ? n_words : 1), -1);
    for (int w = 0; w < n_words; w++) {
        uint32_t k[8];
        int len;
        rec_key(dict + (size_t)w * 32, k, &len);
        if (len == 0) continue;
        std::string key((const char*)dict + (size_t)w * 32, (size_t)len);
        auto it = first.find(key);
        if (it == first.end()) {
            first.emplace(key, w);
            uniq.push_back(w);
            last[(size_t)w] = w;
        } else {
            int h = it->second;
            T.next_dup[(size_t)last[(size_t)h]] = w;
            last[(size_t)h] = w;
        }
    }
    uint32_t nb = (uint32_t)((double)uniq.size() / (GREP_WAYS * 0.85)) + 16u;
    for (int attempt = 0; attempt < 20; attempt++, nb = nb + nb / 8u + 1u) {
        std::vector<int> slot_of(nb * GREP_WAYS, -1);
        uint64_t rng = 0x243F6A8885A308D3ULL ^ nb;
        bool ok = true;
        for (int w : uniq) {
            int cur = w;
            int kicks = 0;
            for (;;) {
                uint32_t k[8];
                int len;
                rec_key(dict + (size_t)cur * 32, k, &len);
                uint64_t h = grep_hash(k, len);
                uint32_t b[2] = {grep_b1(h, nb), grep_b2(h, nb)};
                int placed = -1;
                for (int r = 0; r < 2 && placed < 0; r++)
                    for (int i = 0; i < GREP_WAYS; i++)
                        if (slot_of[b[r] * GREP_WAYS + (uint32_t)i] < 0) { placed = (int)(b[r] * GREP_WAYS + (uint32_t)i); break; }
                if (placed >= 0) {
                    slot_of[(size_t)placed] = cur;
                    break;
                }
                if (++kicks > 2000) { ok = false; break; }
                rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17;
                uint32_t victim = b[rng & 1u] * GREP_WAYS + (uint32_t)((rng >> 8) & 3u);
                int ev = slot_of[victim];
                slot_of[victim] = cur;
                cur = ev;
            }
            if (!ok) break;
        }
        if (!ok) continue;
        T.nb = nb;
        T.tbl.assign(nb * GREP_WAYS, 0u);
        T.recs.assign((size_t)nb * GREP_WAYS * 8, 0u);
        T.slot_word.assign(nb * GREP_WAYS, 0xFFFFFFFFu);
        for (uint32_t s = 0; s < nb * GREP_WAYS; s++) {
            int w = slot_of[s];
            if (w < 0) continue;
            uint32_t k[8];
            int len;
            rec_key(dict + (size_t)w * 32, k, &len);
            uint64_t h = grep_hash(k, len);
            T.tbl[s] = grep_tag(h) << GREP_TAG_SHIFT;
            memcpy(&T.recs[(size_t)s * 8], k, 32);
            T.slot_word[s] = (uint32_t)w;
        }
        return true;
    }
    return false;
}

} // namespace

struct gfs_grep {
    gfs_ctx* ctx = nullptr;
    int n_files = 0, n_words = 0;
    HostTable T;
    GrepDev dev{};
    void* dmem = nullptr; /* one allocation for everything */
    std::vector<uint64_t> sizes;
    bool smem = true;
    size_t smem_bytes = 0;
    int sms = 0;
    uint32_t last_status[2] = {0, 0};
};

/* Data pages per window so that all CTAs' windows fit in half the pool. */
static void set_window(gfs_grep* g, int n_ctas) {
    uint32_t frames = gfs_num_frames(g->ctx);
    uint64_t per = (uint64_t)frames / 2u / (uint64_t)(n_ctas > 0 ? n_ctas : 1);
    uint32_t w = per > 2u ? (uint32_t)(per - 2u) : 1u;
    g->dev.win_data = w > GR_WIN - 2 ? GR_WIN - 2 : w;
}

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

extern "C" {

void gfs__preload_grep() {
    cudaFuncAttributes a;
    cudaFuncGetAttributes(&a, k_grep_scan<true>);
    cudaFuncGetAttributes(&a, k_grep_scan<false>);
    cudaFuncGetAttributes(&a, k_grep_fixup);
    cudaFuncGetAttributes(&a, k_open_files);
    cudaFuncGetAttributes(&a, k_close_files);
}

int gfs_grep_open(gfs_ctx* ctx, const char* dict_path, const char* const* paths, int n_files, gfs_grep** out) {
    *out = nullptr;
    if (n_files < 1 || !dict_path) return -GFS_EINVAL;
    for (int i = 0; i < n_files; i++)
        if (!paths[i] || strlen(paths[i]) >= GFS_NAME_MAX) return -GFS_EINVAL;
    if (gfs__activate(ctx)) return -GFS_EIO;
    int fd = open(dict_path, O_RDONLY | O_CLOEXEC);
    if (fd < 0) return -errno;
    struct stat st;
    if (fstat(fd, &st) != 0) { close(fd); return -errno; }
    std::vector<uint8_t> dict((size_t)st.st_size + 32, 0);
    ssize_t got = 0;
    while (got < st.st_size) {
        ssize_t r = pread(fd, dict.data() + got, (size_t)(st.st_size - got), got);
        if (r <= 0) break;
        got += r;
    }
    close(fd);
    gfs_grep* g = new gfs_grep();
    g->ctx = ctx;
    g->n_files = n_files;
    g->n_words = (int)(st.st_size / 32); /* grep_text_gpu.cu:221 */
    if (!build_table(dict.data(), g->n_words, g->T)) { delete g; return -GFS_ENOMEM; }
    const uint32_t nb = g->T.nb;
    /* device layout */
    size_t o_tbl = 0, o_recs = align_up(o_tbl + (size_t)nb * 16, 256), o_sw = align_up(o_recs + (size_t)nb * 4 * 32, 256),
           o_nd = align_up(o_sw + (size_t)nb * 16, 256), o_cnt = align_up(o_nd + (size_t)g->n_words * 4 + 4, 256),
           o_fds = align_up(o_cnt + (size_t)g->n_words * n_files * 4 + 4, 256), o_sz = align_up(o_fds + (size_t)n_files * 4, 256),
           o_pf = align_up(o_sz + (size_t)n_files * 8, 256), o_fl = align_up(o_pf + (size_t)(n_files + 1) * 8, 256),
           o_st = align_up(o_fl + (size_t)n_files * 4, 256), o_names = align_up(o_st + 64, 256),
           total = align_up(o_names + (size_t)n_files * GFS_NAME_MAX, 256);
    if (cudaMalloc(&g->dmem, total) != cudaSuccess) { delete g; return -GFS_ENOMEM; }
    uint8_t* b = (uint8_t*)g->dmem;
    cudaMemset(b, 0, total);
    cudaMemcpy(b + o_tbl, g->T.tbl.data(), (size_t)nb * 16, cudaMemcpyHostToDevice);
    cudaMemcpy(b + o_recs, g->T.recs.data(), (size_t)nb * 4 * 32, cudaMemcpyHostToDevice);
    cudaMemcpy(b + o_sw, g->T.slot_word.data(), (size_t)nb * 16, cudaMemcpyHostToDevice);
    if (g->n_words) cudaMemcpy(b + o_nd, g->T.next_dup.data(), (size_t)g->n_words * 4, cudaMemcpyHostToDevice);
    std::vector<char> names((size_t)n_files * GFS_NAME_MAX, 0);
    for (int i = 0; i < n_files; i++) memcpy(&names[(size_t)i * GFS_NAME_MAX], paths[i], strlen(paths[i]));
    cudaMemcpy(b + o_names, names.data(), names.size(), cudaMemcpyHostToDevice);
    GrepDev& d = g->dev;
    d.n_files = n_files;
    d.n_words = g->n_words;
    d.fds = (const int*)(b + o_fds);
    d.sizes = (const uint64_t*)(b + o_sz);
    d.chunk_prefix = (const uint64_t*)(b + o_pf);
    d.nb = nb;
    d.table = (const uint32_t*)(b + o_tbl);
    d.recs = (const uint4*)(b + o_recs);
    d.slot_word = (const uint32_t*)(b + o_sw);
    d.next_dup = (const int32_t*)(b + o_nd);
    d.counts = (uint32_t*)(b + o_cnt);
    d.long_flags = (uint32_t*)(b + o_fl);
    d.status = (uint32_t*)(b + o_st);
    cudaStream_t s = (cudaStream_t)gfs_kernel_stream(ctx);
    k_open_files<<<n_files, 128, 0, s>>>((const char*)(b + o_names), n_files, (int*)d.fds, (uint64_t*)d.sizes);
    if (cudaStreamSynchronize(s) != cudaSuccess) { gfs_grep_close(g); return -GFS_EIO; }
    std::vector<int> fds((size_t)n_files);
    g->sizes.resize((size_t)n_files);
    cudaMemcpy(fds.data(), d.fds, (size_t)n_files * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(g->sizes.data(), d.sizes, (size_t)n_files * 8, cudaMemcpyDeviceToHost);
    for (int i = 0; i < n_files; i++)
        if (fds[(size_t)i] < 0) {
            int e = fds[(size_t)i];
            gfs_grep_close(g);
            return e;
        }
    std::vector<uint64_t> pf((size_t)n_files + 1, 0);
    for (int i = 0; i < n_files; i++) pf[(size_t)i + 1] = pf[(size_t)i] + (g->sizes[(size_t)i] + GR_CH - 1) / GR_CH;
    cudaMemcpy((void*)d.chunk_prefix, pf.data(), pf.size() * 8, cudaMemcpyHostToDevice);
    d.total_chunks = pf[(size_t)n_files];
    /* shared memory: table (if it fits) + stages + token lists + scratch */
    int dev = 0, sms = 0, maxsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    g->sms = sms;
    size_t fixed = (size_t)GR_STAGES * (GR_CH + 96) + (size_t)GR_WARPS * 2 * GR_LIST * 2 + (size_t)GR_WARPS * 48 + 256;
    size_t with_tbl = align_up((size_t)nb * 16, 128) + fixed;
    g->smem = with_tbl <= (size_t)maxsm;
    g->smem_bytes = g->smem ? with_tbl : fixed;
    cudaFuncSetAttribute(k_grep_scan<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)with_tbl);
    cudaFuncSetAttribute(k_grep_scan<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fixed);
    *out = g;
    return 0;
}

int gfs_grep_run(gfs_grep* g, int n_ctas, float* kernel_ms) {
    if (!g) return -GFS_EINVAL;
    if (gfs__activate(g->ctx)) return -GFS_EIO;
    cudaStream_t s = (cudaStream_t)gfs_kernel_stream(g->ctx);
    GrepDev& d = g->dev;
    cudaMemsetAsync(d.counts, 0, (size_t)g->n_words * g->n_files * 4, s);
    cudaMemsetAsync(d.long_flags, 0, (size_t)g->n_files * 4, s);
    cudaMemsetAsync(d.status, 0, 8, s);
    if (n_ctas <= 0) n_ctas = g->sms;
    set_window(g, n_ctas);
    cudaEvent_t a, b;
    if (kernel_ms) {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, s);
    }
    if (g->smem) k_grep_scan<true><<<n_ctas, GR_THREADS, g->smem_bytes, s>>>((gfs_state*)gfs_device_state(g->ctx), d);
    else k_grep_scan<false><<<n_ctas, GR_THREADS, g->smem_bytes, s>>>((gfs_state*)gfs_device_state(g->ctx), d);
    cudaError_t le = cudaGetLastError();
    k_grep_fixup<<<g->n_files, 32, 0, s>>>((gfs_state*)gfs_device_state(g->ctx), d);
    if (kernel_ms) {
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(kernel_ms, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    cudaError_t e = cudaStreamSynchronize(s);
    if (le != cudaSuccess || e != cudaSuccess) {
        fprintf(stderr, "gpufs_gb300: grep kernel failed: %s\n", cudaGetErrorString(le != cudaSuccess ? le : e));
        return -GFS_EIO;
    }
    uint32_t status[2] = {0, 0};
    cudaMemcpy(status, d.status, 8, cudaMemcpyDeviceToHost);
    g->last_status[0] = status[0];
    g->last_status[1] = status[1];
    return status[0] ? -((status[0] & GFS_ERRB_TIMEOUT) ? GFS_ETIMEDOUT : GFS_EIO) : 0;
}

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
    std::vector<cudaEvent_t> ev((size_t)steps * 2 + 2);
    for (auto& e : ev) cudaEventCreate(&e);
    cudaMemsetAsync(d.status, 0, 8, s);
    set_window(g, n_ctas);
    cudaEventRecord(ev[0], s);
    for (int i = 0; i < steps; i++) {
        cudaMemsetAsync(d.counts, 0, (size_t)g->n_words * g->n_files * 4, s);
        cudaMemsetAsync(d.long_flags, 0, (size_t)g->n_files * 4, s);
        cudaEventRecord(ev[2 + 2 * (size_t)i], s);
        if (g->smem) k_grep_scan<true><<<n_ctas, GR_THREADS, g->smem_bytes, s>>>(S, d);
        else k_grep_scan<false><<<n_ctas, GR_THREADS, g->smem_bytes, s>>>(S, d);
        cudaEventRecord(ev[3 + 2 * (size_t)i], s);
        k_grep_fixup<<<g->n_files, 32, 0, s>>>(S, d);
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

int gfs_grep_counts(gfs_grep* g, uint32_t* host_counts) {
    if (!g) return -GFS_EINVAL;
    cudaStream_t s = (cudaStream_t)gfs_kernel_stream(g->ctx);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -GFS_EIO;
    return cudaMemcpy(host_counts, g->dev.counts, (size_t)g->n_words * g->n_files * 4, cudaMemcpyDeviceToHost) ==
                   cudaSuccess
               ? 0
               : -GFS_EIO;
}

int gfs_grep_info(gfs_grep* g, long long* out, int n) {
    long long v[8] = {g->n_words, g->n_files, (long long)g->T.nb, g->smem ? 1 : 0, (long long)g->smem_bytes,
                      (long long)g->dev.total_chunks, (long long)g->last_status[0], (long long)g->last_status[1]};
    int k = n < 8 ? n : 8;
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
        int* rcs = nullptr;
        if (cudaMalloc(&rcs, (size_t)g->n_files * 4) == cudaSuccess) {
            k_close_files<<<g->n_files, 128, 0, s>>>(g->dev.fds, g->n_files, rcs);
            cudaStreamSynchronize(s);
            std::vector<int> h((size_t)g->n_files);
            cudaMemcpy(h.data(), rcs, h.size() * 4, cudaMemcpyDeviceToHost);
            for (int x : h)
                if (x < 0 && !rc) rc = x;
            cudaFree(rcs);
        }
    }
    cudaFree(g->dmem);
    delete g;
    return rc;
}

int gfs_grep_text(gfs_ctx* ctx, const char* dict_path, const char* const* paths, int n_files, uint32_t* host_counts,
                  int n_ctas) {
    gfs_grep* g = nullptr;
    int rc = gfs_grep_open(ctx, dict_path, paths, n_files, &g);
    if (rc) return rc;
    rc = gfs_grep_run(g, n_ctas, nullptr);
    if (!rc) rc = gfs_grep_counts(g, host_counts);
    int c = gfs_grep_close(g);
    return rc ? rc : c;
}

} /* extern "C" */

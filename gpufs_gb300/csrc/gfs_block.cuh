/*
 * Block- and warp-collective file operations (the bodies behind the
 * reference-named device API).  Every thread of the calling block (warp for
 * the _warp forms) must call with the same arguments, as in the reference
 * (libgpufs/fs_calls.cu:685-687: "pread is expected to be issued by all
 * threads in a thread block with the same parameters").
 *
 *   blk_read   <- gread        fs_calls.cu:689-737
 *   blk_write  <- gwrite       fs_calls.cu:739-802
 *   blk_mmap   <- gmmap        fs_calls.cu:422-481
 *   blk_munmap <- gmunmap      fs_calls.cu:385-401
 *   blk_flush  <- gfsync/flush fs_calls.cu:107-125, fs_structures.cu:263-298
 *   blk_close  <- gclose       fs_calls.cu:35-105
 *
 * GB300 changes: up to 32 pages of one request are faulted in parallel, one
 * lane per page; missed pages of a file with a registered host mapping are
 * filled by the whole block from the mapping (SM loads over the host link,
 * no request to the host), others by the host in parallel; then all threads
 * copy with 16-byte vectors.  gmmap fills a missed page the same way.
 * Dirty pages are staged for write-back by the closing block's warps.
 * Reads clamp at end of file and return the byte count (the reference
 * returns `size` whatever it read).
 */
#ifndef GFS_BLOCK_CUH
#define GFS_BLOCK_CUH

#include "gfs_device.cuh"

namespace gfsd {
namespace { /* internal linkage: every TU gets its own copy */

__device__ __forceinline__ int blk_tid() {
    return threadIdx.x + threadIdx.y * blockDim.x + threadIdx.z * blockDim.x * blockDim.y;
}
__device__ __forceinline__ int blk_nthr() { return blockDim.x * blockDim.y * blockDim.z; }

/* group copy: threads [rank] of a group of `gsize` (<= 32, one warp) */
__device__ __forceinline__ void grp_copy(uint8_t* dst, const uint8_t* src, size_t n, int rank, int gsize) {
    if (gsize == 32) { warp_copy(dst, src, n, rank); return; }
    for (size_t k = (size_t)rank; k < n; k += (size_t)gsize) dst[k] = src[k];
}
__device__ __forceinline__ void grp_zero(uint8_t* dst, size_t n, int rank, int gsize) {
    if (gsize == 32) { warp_zero(dst, n, rank); return; }
    for (size_t k = (size_t)rank; k < n; k += (size_t)gsize) dst[k] = 0;
}

/* Copy a round of `npages` pages' bytes [pos, end) between frames and a
 * linear user buffer (frames[j] holds page first + j); to_frame selects the
 * direction.  Every warp takes an equal contiguous slice of the round (cut
 * at 512-byte multiples, so frame and buffer keep their relative alignment)
 * and walks the page boundaries inside it: a round whose first and last
 * pages are partial keeps all warps equally busy. */
__device__ __forceinline__ void blk_copy_round(gfs_state* S, const int* frames, uint32_t first, int npages,
                                               uint64_t pos, uint64_t end, uint8_t* ubuf, uint64_t ubase,
                                               bool to_frame) {
    const int tid = blk_tid(), nthr = blk_nthr();
    const int warp = tid >> 5, lane = tid & 31;
    const int nwarps = (nthr + 31) >> 5;
    const int gsize = (warp == nwarps - 1) ? (nthr - 32 * warp) : 32;
    const uint32_t lp = S->log_page;
    (void)npages;
    if (end <= pos) return;
    const uint64_t pmask = (1ull << lp) - 1u;
    const uintptr_t delta = (uintptr_t)ubuf - (uintptr_t)ubase; /* user address of file offset x: delta + x */
    const bool ug = __isGlobal(ubuf) != 0; /* the user buffer may be a block's shared memory */
    if ((delta & 15u) == 0u) {
        /* frame and buffer agree mod 16 (frames are page-aligned): the whole
         * block sweeps the round as one stream of 16-byte units, consecutive
         * threads on consecutive units, four in flight per thread -- one
         * DRAM stream per block instead of one per warp */
        const uint64_t u0 = (pos + 15u) >> 4, u1 = end >> 4;
        if (u0 >= u1) {
            for (uint64_t x = pos + (uint64_t)tid; x < end; x += (uint64_t)nthr) {
                uint8_t* f = frame_data(S, (uint32_t)frames[(uint32_t)(x >> lp) - first]) + (x & pmask);
                uint8_t* u = (uint8_t*)(delta + x);
                if (to_frame) *f = *u;
                else *u = *f;
            }
            return;
        }
        /* bytes before the first and after the last whole unit */
        for (uint64_t x = pos + (uint64_t)tid; x < (u0 << 4); x += (uint64_t)nthr) {
            uint8_t* f = frame_data(S, (uint32_t)frames[(uint32_t)(x >> lp) - first]) + (x & pmask);
            uint8_t* u = (uint8_t*)(delta + x);
            if (to_frame) *f = *u;
            else *u = *f;
        }
        for (uint64_t x = (u1 << 4) + (uint64_t)tid; x < end; x += (uint64_t)nthr) {
            uint8_t* f = frame_data(S, (uint32_t)frames[(uint32_t)(x >> lp) - first]) + (x & pmask);
            uint8_t* u = (uint8_t*)(delta + x);
            if (to_frame) *f = *u;
            else *u = *f;
        }
        const uint64_t step = (uint64_t)nthr;
        uint64_t u = u0 + (uint64_t)tid;
        for (; u + 3 * step < u1; u += 4 * step) {
            uint4* fp[4];
            uint4* up[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const uint64_t x = (u + (uint64_t)k * step) << 4;
                fp[k] = (uint4*)(frame_data(S, (uint32_t)frames[(uint32_t)(x >> lp) - first]) + (x & pmask));
                up[k] = (uint4*)(delta + x);
            }
            uint4 v[4];
            if (to_frame) {
#pragma unroll
                for (int k = 0; k < 4; k++) v[k] = ld_user4(up[k], ug);
#pragma unroll
                for (int k = 0; k < 4; k++) *fp[k] = v[k];
            } else {
#pragma unroll
                for (int k = 0; k < 4; k++) v[k] = ld_cg4(fp[k]);
#pragma unroll
                for (int k = 0; k < 4; k++) *up[k] = v[k];
            }
        }
        for (; u < u1; u += step) {
            const uint64_t x = u << 4;
            uint4* f = (uint4*)(frame_data(S, (uint32_t)frames[(uint32_t)(x >> lp) - first]) + (x & pmask));
            uint4* up = (uint4*)(delta + x);
            if (to_frame) *f = ld_user4(up, ug);
            else *up = ld_cg4(f);
        }
        return;
    }
    const uint64_t per = ((end - pos + (uint64_t)nwarps - 1) / (uint64_t)nwarps + 511u) & ~511ull;
    uint64_t a = pos + (uint64_t)warp * per;
    const uint64_t b = a + per < end ? a + per : end;
    while (a < b) {
        const uint32_t j = (uint32_t)(a >> lp) - first;
        const uint64_t pstart = (uint64_t)(first + j) << lp;
        const uint64_t e = b < pstart + (1ull << lp) ? b : pstart + (1ull << lp);
        uint8_t* fptr = frame_data(S, (uint32_t)frames[j]) + (a - pstart);
        uint8_t* uptr = ubuf + (a - ubase);
        if (to_frame) grp_copy(fptr, uptr, e - a, lane, gsize);
        else grp_copy(uptr, fptr, e - a, lane, gsize);
        a = e;
    }
}

/* ------------------------------------------------------------------ */
/* read                                                                */
/* ------------------------------------------------------------------ */
/* Fill the fresh frames of a round (bit j of `fresh`: frames[j] holds page
 * first + j, still LOADING) from the file's registered host mapping: the
 * whole block sweeps each page in turn, consecutive threads on consecutive
 * 16-byte units (the mapping is page aligned), four loads in flight per
 * thread, so a block keeps its threads x 64 bytes in flight over the host
 * link. */
__device__ __forceinline__ void blk_fill_round(gfs_state* S, const int* frames, unsigned fresh, uint32_t first,
                                               uint64_t map_dev, uint64_t fsize) {
    const uint64_t tid = (uint64_t)blk_tid(), nthr = (uint64_t)blk_nthr();
    const uint32_t lp = S->log_page;
    for (unsigned m = fresh; m; m &= m - 1u) {
        const int j = __ffs(m) - 1;
        const uint64_t pst = ((uint64_t)(first + (uint32_t)j)) << lp;
        uint8_t* dst = frame_data(S, (uint32_t)frames[j]);
        if (!map_dev || pst >= fsize) {
            /* no bytes behind the page (a fresh page without a mapping, or
             * past the end of the file): hand out zeros */
            for (uint64_t i = tid; i < ((1ull << lp) >> 4); i += nthr) ((uint4*)dst)[i] = make_uint4(0, 0, 0, 0);
            continue;
        }
        const uint64_t len = fsize - pst < (1ull << lp) ? fsize - pst : (1ull << lp);
        const uint4* src = (const uint4*)(uintptr_t)(map_dev + pst);
        uint4* d4 = (uint4*)dst;
        const uint64_t n16 = len >> 4;
        uint64_t i = tid;
        for (; i + 3u * nthr < n16; i += 4u * nthr) {
            const uint4 a = src[i], b = src[i + nthr], c = src[i + 2u * nthr], d = src[i + 3u * nthr];
            d4[i] = a;
            d4[i + nthr] = b;
            d4[i + 2u * nthr] = c;
            d4[i + 3u * nthr] = d;
        }
        for (; i < n16; i += nthr) d4[i] = src[i];
        const uint8_t* s1 = (const uint8_t*)src;
        for (uint64_t q = (n16 << 4) + tid; q < len; q += nthr) dst[q] = s1[q];
    }
}

__device__ __noinline__ long long blk_read(gfs_state* S, int fd, uint64_t off, uint64_t size, uint8_t* buf) {
    __shared__ PinFile s_pf;
    __shared__ uint64_t s_off, s_size;
    __shared__ uint8_t* s_buf;
    __shared__ int s_frames[32];
    __shared__ unsigned s_fresh, s_later;
    __shared__ int s_err, s_round, s_retry;
    const int tid = blk_tid(), nthr = blk_nthr();
    const unsigned m0 = nthr >= 32 ? 0xFFFFFFFFu : ((1u << nthr) - 1u); /* lanes of warp 0 */
    __syncthreads();
    if (tid == 0) {
        s_err = 0;
        s_round = nthr < 32 ? nthr : 32;
        if (fd < 0 || (uint32_t)fd >= S->n_files || sstatus(ld_acq(&S->files[fd].st)) != GFS_SS_OPEN) {
            s_err = -GFS_EBADF;
        } else {
            s_pf = pin_file(S, fd);
            uint64_t fsz = s_pf.size;
            s_size = off >= fsz ? 0 : (size < fsz - off ? size : fsz - off);
        }
        s_off = off;
        s_buf = buf;
    }
    __syncthreads();
    if (s_err) return s_err;
    const uint64_t total = s_size, base = s_off;
    const uint32_t lp = S->log_page;
    uint64_t done = 0;
    while (done < total) {
        const uint64_t pos = base + done;
        const uint32_t first = (uint32_t)(pos >> lp);
        const uint32_t last = (uint32_t)((base + total - 1) >> lp);
        int npages = (int)(last - first + 1u);
        if (npages > s_round) npages = s_round;
        if (tid < 32) {
            int r = 0;
            bool fresh = false;
            if (tid < npages) {
                /* a miss of a file with a registered mapping is filled by
                 * this block (SM loads over the host link); others by the
                 * host */
                r = pin_page(S, s_pf, first + (uint32_t)tid,
                             GFS_PIN_READ | GFS_PIN_SMFILL | (npages > 1 ? GFS_PIN_NOALLOC : 0), &fresh);
                s_frames[tid] = r;
            }
            const unsigned fr_mask = __ballot_sync(m0, tid < npages && r >= 0 && fresh);
            unsigned nomem = __ballot_sync(m0, tid < npages && r == -GFS_ENOMEM);
            unsigned bad = __ballot_sync(m0, tid < npages && r < 0 && r != -GFS_ENOMEM && r != -GFS_EAGAIN);
            const unsigned later = __ballot_sync(m0, tid < npages && r == -GFS_EAGAIN);
            if (bad || nomem) {
                if (tid < npages && r >= 0) {
                    if (fresh) { /* give back a page never filled */
                        gfs_frame* F = &S->frames[r];
                        index_remove(S, ld_rlx64(&F->key), (uint32_t)r);
                        release_owned(S, (uint32_t)r, GFS_FS_LOADING, 1u);
                    } else {
                        unpin(S, (uint32_t)r);
                    }
                }
                int e = bad ? __shfl_sync(m0, r, __ffs(bad) - 1) : 0;
                if (tid == 0) {
                    s_retry = 1;
                    if (bad) s_err = e;
                    else if (npages == 1) s_err = -GFS_ENOMEM;
                    s_round = s_round > 1 ? s_round / 2 : 1;
                }
            } else if (tid == 0) {
                s_retry = 0;
                s_fresh = fr_mask;
                s_later = later;
            }
        }
        __syncthreads();
        if (s_err) return s_err;
        if (s_retry) continue;
        if (s_fresh) {
            blk_fill_round(S, s_frames, s_fresh, first, s_pf.map_dev, s_pf.size);
            __syncthreads();
            if (tid < npages && ((s_fresh >> tid) & 1u)) {
                const uint64_t pst = ((uint64_t)(first + (uint32_t)tid)) << lp;
                const uint64_t len = !s_pf.map_dev || pst >= s_pf.size ? 0u
                                     : (s_pf.size - pst < (1ull << lp) ? s_pf.size - pst : (1ull << lp));
                st_rlx(&S->frames[s_frames[tid]].content, (uint32_t)len);
                publish_valid(S, (uint32_t)s_frames[tid]);
            }
        }
        if (s_later) {
            /* pages another block was loading: now that every page this
             * block filled is published, wait for them (a miss by then is
             * filled by the host inside pin_page) */
            __syncthreads();
            if (tid < npages && ((s_later >> tid) & 1u)) {
                bool fresh = false;
                int r = pin_page(S, s_pf, first + (uint32_t)tid, GFS_PIN_READ, &fresh);
                if (r >= 0 && fresh) { /* no bytes behind it: zeros */
                    uint32_t* d = (uint32_t*)frame_data(S, (uint32_t)r);
                    for (uint32_t k = 0; k < (S->page_size >> 2); k++) d[k] = 0u;
                    publish_valid(S, (uint32_t)r);
                }
                s_frames[tid] = r;
                if (r < 0) atomicCAS(&s_err, 0, r);
            }
            __syncthreads();
            if (s_err) {
                /* give back the pages held */
                if (tid < npages && s_frames[tid] >= 0) unpin(S, (uint32_t)s_frames[tid]);
                __syncthreads();
                return s_err;
            }
        }
        uint64_t pend = ((uint64_t)(first + (uint32_t)npages)) << lp;
        uint64_t end = base + total < pend ? base + total : pend;
        blk_copy_round(S, s_frames, first, npages, pos, end, s_buf, base, false);
        __syncthreads();
        if (tid < npages) unpin(S, (uint32_t)s_frames[tid]);
        if (tid == 0) count(S, &S->stats.hits, (unsigned long long)npages);
        done = end - base;
        __syncthreads();
    }
    return (long long)total;
}

/* ------------------------------------------------------------------ */
/* write                                                               */
/* ------------------------------------------------------------------ */
__device__ __noinline__ long long blk_write(gfs_state* S, int fd, uint64_t off, uint64_t size, const uint8_t* buf) {
    __shared__ PinFile s_pf;
    __shared__ uint64_t s_off, s_size;
    __shared__ const uint8_t* s_buf;
    __shared__ int s_frames[32];
    __shared__ unsigned s_fresh;
    __shared__ int s_err, s_round, s_retry;
    const int tid = blk_tid(), nthr = blk_nthr();
    const unsigned m0 = nthr >= 32 ? 0xFFFFFFFFu : ((1u << nthr) - 1u); /* lanes of warp 0 */
    __syncthreads();
    if (tid == 0) {
        s_err = 0;
        s_round = nthr < 32 ? nthr : 32;
        if (fd < 0 || (uint32_t)fd >= S->n_files || sstatus(ld_acq(&S->files[fd].st)) != GFS_SS_OPEN) {
            s_err = -GFS_EBADF;
        } else {
            s_pf = pin_file(S, fd);
            if (s_pf.oflags == O_GRDONLY) s_err = -GFS_EBADF;
        }
        s_off = off;
        s_size = size;
        s_buf = buf;
    }
    __syncthreads();
    if (s_err) return s_err;
    const uint64_t total = s_size, base = s_off;
    const uint32_t lp = S->log_page;
    const uint64_t page = 1ull << lp;
    uint64_t done = 0;
    while (done < total) {
        const uint64_t pos = base + done;
        const uint32_t first = (uint32_t)(pos >> lp);
        const uint32_t last = (uint32_t)((base + total - 1) >> lp);
        int npages = (int)(last - first + 1u);
        if (npages > s_round) npages = s_round;
        if (tid < 32) {
            int r = 0;
            bool fresh = false;
            if (tid < npages) {
                uint64_t pst = ((uint64_t)(first + (uint32_t)tid)) << lp;
                bool full = pos <= pst && base + total >= pst + page;
                int mode = full ? GFS_PIN_WFULL : (s_pf.oflags == O_GWRONCE ? GFS_PIN_WONCE : GFS_PIN_WPART);
                r = pin_page(S, s_pf, first + (uint32_t)tid, mode | (npages > 1 ? GFS_PIN_NOALLOC : 0), &fresh);
                s_frames[tid] = r;
            }
            unsigned fr_mask = __ballot_sync(m0, tid < npages && r >= 0 && fresh);
            unsigned nomem = __ballot_sync(m0, tid < npages && r == -GFS_ENOMEM);
            unsigned bad = __ballot_sync(m0, tid < npages && r < 0 && r != -GFS_ENOMEM);
            if (bad || nomem) {
                if (tid < npages && r >= 0) {
                    if (fresh) { /* give back a page we never initialised */
                        gfs_frame* F = &S->frames[r];
                        uint64_t k = ld_rlx64(&F->key);
                        index_remove(S, k, (uint32_t)r);
                        release_owned(S, (uint32_t)r, GFS_FS_LOADING, 1u);
                    } else {
                        unpin(S, (uint32_t)r);
                    }
                }
                int e = bad ? __shfl_sync(m0, r, __ffs(bad) - 1) : 0;
                if (tid == 0) {
                    s_retry = 1;
                    if (bad) s_err = e;
                    else if (npages == 1) s_err = -GFS_ENOMEM;
                    s_round = s_round > 1 ? s_round / 2 : 1;
                }
            } else if (tid == 0) {
                s_retry = 0;
                s_fresh = fr_mask;
            }
        }
        __syncthreads();
        if (s_err) return s_err;
        if (s_retry) continue;
        uint64_t pend = ((uint64_t)(first + (uint32_t)npages)) << lp;
        uint64_t end = base + total < pend ? base + total : pend;
        /* zero the uncovered parts of fresh pages */
        if (s_fresh) {
            const int warp = tid >> 5, lane = tid & 31, nwarps = (nthr + 31) >> 5;
            const int gsize = (warp == nwarps - 1) ? (nthr - 32 * warp) : 32;
            for (int j = warp; j < npages; j += nwarps) {
                if (!((s_fresh >> j) & 1u)) continue;
                uint64_t pst = ((uint64_t)(first + (uint32_t)j)) << lp;
                uint64_t a = pos > pst ? pos - pst : 0;
                uint64_t b = end < pst + page ? end - pst : page;
                uint8_t* d = frame_data(S, (uint32_t)s_frames[j]);
                if (a) grp_zero(d, a, lane, gsize);
                if (b < page) grp_zero(d + b, page - b, lane, gsize);
            }
        }
        blk_copy_round(S, s_frames, first, npages, pos, end, (uint8_t*)s_buf, base, true);
        __syncthreads();
        if (tid < npages) {
            uint32_t fr = (uint32_t)s_frames[tid];
            uint64_t pst = ((uint64_t)(first + (uint32_t)tid)) << lp;
            uint64_t b = end < pst + page ? end - pst : page;
            atomicMax(&S->frames[fr].content, (uint32_t)b);
            if ((s_fresh >> tid) & 1u) publish_valid(S, fr);
            mark_dirty(S, fr);
            unpin(S, fr);
        }
        if (tid == 0) atomicMax((unsigned long long*)&S->files[s_pf.slot].size, (unsigned long long)end);
        done = end - base;
        __syncthreads();
    }
    return (long long)total;
}

/* ------------------------------------------------------------------ */
/* map / unmap                                                         */
/* ------------------------------------------------------------------ */
__device__ __forceinline__ int mmap_mode(int oflags) {
    if (oflags == O_GRDONLY) return GFS_PIN_READ;
    if (oflags == O_GWRONCE) return GFS_PIN_WONCE;
    return GFS_PIN_WPART;
}

/* Single-thread part of a mapping: pin the page holding `off`.  Returns the
 * frame or -error; *fresh when the caller must fill (or zero) and publish it.
 * fill (optional): for a read-only file with a registered host mapping a
 * missed page comes back fresh with fill->len > 0: the caller's threads copy
 * the page's fill->len bytes from the mapping (fill->map, page fill->blk;
 * no host request).  The caller holds no other unfilled page, so a page
 * another caller is loading is simply waited for.  Without fill, or for
 * other files, fill->len is 0 and a fresh page is zeroed. */
struct MapFill {
    uint64_t map, size, len;
    uint32_t blk;
};
__device__ __forceinline__ int map_pin(gfs_state* S, int fd, uint64_t off, uint64_t size, bool* fresh, int ref,
                                       MapFill* fill = nullptr) {
    *fresh = false;
    if (fill) fill->len = 0;
    if (fd < 0 || (uint32_t)fd >= S->n_files || sstatus(ld_acq(&S->files[fd].st)) != GFS_SS_OPEN) return -GFS_EBADF;
    PinFile pf = pin_file(S, fd);
    const uint64_t page = (uint64_t)S->page_size;
    uint64_t boff = off & (page - 1);
    if (boff + size > page) { set_error(S, GFS_ERRB_ARG); return -GFS_EINVAL; }
    if (pf.oflags == O_GRDONLY && off >= pf.size) return -GFS_EINVAL;
    const uint32_t blk = (uint32_t)(off >> S->log_page);
    const bool smfill = fill && pf.oflags == O_GRDONLY && pf.map_dev;
    int r = pin_page(S, pf, blk, mmap_mode(pf.oflags) | (smfill ? GFS_PIN_SMFILL : 0), fresh);
    if (r == -GFS_EAGAIN) r = pin_page(S, pf, blk, mmap_mode(pf.oflags), fresh);
    if (r < 0) return r;
    if (*fresh && smfill) {
        const uint64_t pst = (uint64_t)blk << S->log_page;
        fill->map = pf.map_dev;
        fill->size = pf.size;
        fill->blk = blk;
        fill->len = pf.size - pst < page ? pf.size - pst : page;
    }
    if (ref > 1) atomicAdd(&S->frames[r].st, (uint32_t)(ref - 1));
    if (pf.oflags != O_GRDONLY) {
        atomicMax(&S->frames[r].content, (uint32_t)(boff + size));
        atomicMax((unsigned long long*)&S->files[fd].size, (unsigned long long)(off + size));
    }
    return r;
}

/* Block-collective: make a fresh frame returned by map_pin valid -- its
 * bytes copied from the file's mapping (fill.len > 0) or zeros -- and
 * publish it.  *frame is in shared memory. */
__device__ __forceinline__ void blk_fill_fresh(gfs_state* S, int* frame, const MapFill& fill) {
    const int tid = blk_tid(), nthr = blk_nthr();
    const uint32_t r = (uint32_t)*frame;
    uint8_t* d = frame_data(S, r);
    const uint64_t len = fill.len, l16 = (len + 15u) & ~15ull;
    if (len) blk_fill_round(S, frame, 1u, fill.blk, fill.map, fill.size);
    /* the rest of the page (all of it without a fill) reads as zeros */
    for (uint64_t k = len + (uint64_t)tid; k < l16; k += (uint64_t)nthr) d[k] = 0;
    for (uint64_t k = l16 + 16u * (uint64_t)tid; k < S->page_size; k += 16u * (uint64_t)nthr)
        *(uint4*)(d + k) = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    if (tid == 0) {
        if (len) st_rlx(&S->frames[r].content, (uint32_t)len);
        publish_valid(S, r);
    }
    __syncthreads();
}

__device__ __noinline__ void* blk_mmap(gfs_state* S, int fd, uint64_t off, uint64_t size) {
    __shared__ int s_r;
    __shared__ bool s_fresh;
    __shared__ MapFill s_fill;
    const int tid = blk_tid(), nthr = blk_nthr();
    __syncthreads();
    if (tid == 0) {
        bool fr;
        s_r = map_pin(S, fd, off, size, &fr, 1, &s_fill);
        s_fresh = fr;
    }
    __syncthreads();
    int r = s_r;
    if (r < 0) return (void*)-1; /* GMAP_FAILED */
    if (s_fresh && s_fill.len) {
        /* a missed page of a mapped file: the block copies it from the
         * mapping */
        blk_fill_fresh(S, &s_r, s_fill);
    } else if (s_fresh) {
        const int warp = tid >> 5, lane = tid & 31, nwarps = (nthr + 31) >> 5;
        const int gsize = (warp == nwarps - 1) ? (nthr - 32 * warp) : 32;
        uint64_t chunk = ((uint64_t)S->page_size / (uint64_t)nwarps + 15u) & ~15ull;
        uint64_t a = (uint64_t)warp * chunk;
        if (a < S->page_size) {
            uint64_t b = a + chunk < S->page_size ? a + chunk : S->page_size;
            grp_zero(frame_data(S, (uint32_t)r) + a, b - a, lane, gsize);
        }
        __syncthreads();
        if (tid == 0) publish_valid(S, (uint32_t)r);
        __syncthreads();
    }
    return frame_data(S, (uint32_t)r) + (off & ((uint64_t)S->page_size - 1));
}

__device__ __forceinline__ int addr_frame(gfs_state* S, const volatile void* addr) {
    uintptr_t a = (uintptr_t)addr, p = (uintptr_t)S->pool;
    if (a < p) return -1;
    uint64_t fr = (uint64_t)(a - p) >> S->log_page;
    if (fr >= S->n_frames) return -1;
    return (int)fr;
}

__device__ __forceinline__ int unmap_one(gfs_state* S, const volatile void* addr, int ref) {
    int fr = addr_frame(S, addr);
    if (fr < 0) return -1;
    uint64_t key = ld_rlx64(&S->frames[fr].key);
    uint32_t f = key_file(key);
    if (f < S->n_files && ld_rlx((const uint32_t*)&S->files[f].flags) != (uint32_t)O_GRDONLY) mark_dirty(S, (uint32_t)fr);
    unpin(S, (uint32_t)fr, (uint32_t)ref);
    return 0;
}

__device__ __noinline__ int blk_munmap(gfs_state* S, const volatile void* addr) {
    __shared__ int s_r;
    __threadfence();
    __syncthreads();
    if (blk_tid() == 0) s_r = unmap_one(S, addr, 1);
    __syncthreads();
    return s_r;
}

/* ------------------------------------------------------------------ */
/* flush / close / open                                                */
/* ------------------------------------------------------------------ */
/* Write back every dirty frame of slot fd, spread over the block's threads
 * (each thread one frame at a time, so the block keeps many write-backs in
 * flight).  Returns 0 or the first error. */
/* Write back every dirty frame of slot fd.  Each warp works in rounds: every
 * lane takes its next dirty frame of the file (lanes own interleaved words
 * of the dirty bitmap) and a write-stage slot; the warp copies the lanes'
 * frames into their slots one after another with coalesced 16-byte stores
 * (host memory over the link), then every lane sends its request, so a
 * block keeps its threads' write-backs in flight and the host only merges
 * and writes.  A frame without a slot is copied by the host.  Returns 0 or
 * the first error. */
__device__ __noinline__ int blk_flush(gfs_state* S, int fd) {
    __shared__ int s_err;
    const int tid = blk_tid(), nthr = blk_nthr();
    const int lane = tid & 31, nwarps = (nthr + 31) >> 5, warp = tid >> 5;
    const unsigned wmask = (warp == nwarps - 1 && (nthr & 31)) ? ((1u << (nthr & 31)) - 1u) : 0xFFFFFFFFu;
    __syncthreads();
    if (tid == 0) s_err = 0;
    __syncthreads();
    gfs_file* fe = &S->files[fd];
    const uint32_t gen = ld_rlx(&fe->gen);
    const int host_fd = (int)ld_rlx((const uint32_t*)&fe->host_fd);
    const int oflags = (int)ld_rlx((const uint32_t*)&fe->flags);
    const uint32_t nwords = (S->n_frames + 31u) >> 5;
    uint32_t w = (uint32_t)tid;
    uint32_t bits = w < nwords ? ld_rlx(&S->dirty_bits[w]) : 0u;
    for (;;) {
        /* this lane's next dirty frame of the file, prepared (pinned) */
        int fr = -1;
        uint64_t key = 0;
        while (fr < 0 && w < nwords) {
            if (!bits) {
                w += (uint32_t)nthr;
                bits = w < nwords ? ld_rlx(&S->dirty_bits[w]) : 0u;
                continue;
            }
            const uint32_t b = (uint32_t)(__ffs(bits) - 1);
            bits &= bits - 1u;
            const uint32_t f = (w << 5) | b;
            if (key_file(ld_rlx64(&S->frames[f].key)) != (uint32_t)fd) continue;
            const int p = flush_prepare(S, f, (uint32_t)fd, gen, &key);
            if (p < 0) atomicCAS(&s_err, 0, p);
            if (p > 0) fr = (int)f;
        }
        const unsigned work = __ballot_sync(wmask, fr >= 0);
        if (!work) break;
        const uint32_t content = fr >= 0 ? ld_rlx(&S->frames[fr].content) : 0u;
        const int slot = fr >= 0 ? wstage_claim(S, (uint32_t)fr, content) : -1;
        /* the warp copies each staged lane's frame into its slot */
        for (unsigned m = __ballot_sync(wmask, slot >= 0); m; m &= m - 1u) {
            const int l = __ffs(m) - 1;
            const int f = __shfl_sync(wmask, fr, l);
            const int k = __shfl_sync(wmask, slot, l);
            const uint32_t n16 = (__shfl_sync(wmask, content, l) + 15u) >> 4;
            const uint4* src = (const uint4*)frame_data(S, (uint32_t)f);
            uint4* dst = (uint4*)(S->wstage + (size_t)k * S->page_size);
            /* eight 16-byte loads in flight per lane, then their stores */
            uint32_t i = (uint32_t)lane;
            for (; i + 7u * 32u < n16; i += 8u * 32u) {
                uint4 v[8];
#pragma unroll
                for (int q = 0; q < 8; q++) v[q] = ld_cg4(src + i + 32u * (uint32_t)q);
#pragma unroll
                for (int q = 0; q < 8; q++) dst[i + 32u * (uint32_t)q] = v[q];
            }
            for (; i < n16; i += 32u) dst[i] = ld_cg4(src + i);
        }
        __threadfence_system();
        __syncwarp(wmask);
        if (fr >= 0) {
            const int rc = flush_finish(S, (uint32_t)fr, writeback_frame(S, (uint32_t)fr, key, host_fd, oflags, slot));
            if (rc < 0) atomicCAS(&s_err, 0, rc);
        }
    }
    __syncthreads();
    return s_err;
}

__device__ __noinline__ int blk_close(gfs_state* S, int fd) {
    __shared__ int s_r;
    __syncthreads();
    if (blk_tid() == 0) s_r = file_close_begin(S, fd);
    __syncthreads();
    int r = s_r;
    if (r <= 0) return r;
    int fl = blk_flush(S, fd);
    __syncthreads();
    if (blk_tid() == 0) {
        int c = file_close_finish(S, fd);
        s_r = fl < 0 ? fl : c;
    }
    __syncthreads();
    return s_r;
}

__device__ __noinline__ int blk_open(gfs_state* S, const char* name, int oflags) {
    __shared__ int s_r;
    __syncthreads();
    if (blk_tid() == 0) s_r = file_open(S, name, oflags);
    __syncthreads();
    return s_r;
}

/* single-thread truncate (reference single_thread_ftruncate, fs_calls.cu:127-140;
 * the reference only supports size 0).  Dirty pages below a non-zero new size
 * are written back first; then every cached page of the file is invalidated. */
__device__ __noinline__ int st_truncate(gfs_state* S, int fd, uint64_t size) {
    if (fd < 0 || (uint32_t)fd >= S->n_files) return -GFS_EBADF;
    gfs_file* fe = &S->files[fd];
    if (sstatus(ld_acq(&fe->st)) != GFS_SS_OPEN) return -GFS_EBADF;
    if (size > 0) {
        uint32_t gen = ld_rlx(&fe->gen);
        int host_fd = (int)ld_rlx((const uint32_t*)&fe->host_fd);
        int oflags = (int)ld_rlx((const uint32_t*)&fe->flags);
        uint32_t nwords = (S->n_frames + 31u) >> 5;
        for (uint32_t w = 0; w < nwords; w++) {
            uint32_t bits = ld_rlx(&S->dirty_bits[w]);
            while (bits) {
                uint32_t b = (uint32_t)(__ffs(bits) - 1);
                bits &= bits - 1u;
                uint32_t fr = (w << 5) | b;
                if (key_file(ld_rlx64(&S->frames[fr].key)) == (uint32_t)fd)
                    flush_frame(S, fr, (uint32_t)fd, gen, host_fd, oflags);
            }
        }
    }
    Req r = {};
    r.op = GFS_OP_TRUNC;
    r.host_fd = (int)ld_rlx((const uint32_t*)&fe->host_fd);
    r.file = (uint32_t)fd;
    r.length = size;
    int rc = rpc_call(S, r, file_done(S, (uint32_t)fd));
    if (rc < 0) return rc;
    atomicAdd(&fe->gen, 1u);
    st_rlx64(&fe->size, size);
    __threadfence();
    return 0;
}

/* single-thread fsync */
__device__ __noinline__ int st_fsync(gfs_state* S, int fd) {
    if (fd < 0 || (uint32_t)fd >= S->n_files) return -GFS_EBADF;
    gfs_file* fe = &S->files[fd];
    uint32_t gen = ld_rlx(&fe->gen);
    int host_fd = (int)ld_rlx((const uint32_t*)&fe->host_fd);
    int oflags = (int)ld_rlx((const uint32_t*)&fe->flags);
    uint32_t nwords = (S->n_frames + 31u) >> 5;
    int err = 0;
    for (uint32_t w = 0; w < nwords; w++) {
        uint32_t bits = ld_rlx(&S->dirty_bits[w]);
        while (bits) {
            uint32_t b = (uint32_t)(__ffs(bits) - 1);
            bits &= bits - 1u;
            uint32_t fr = (w << 5) | b;
            if (key_file(ld_rlx64(&S->frames[fr].key)) == (uint32_t)fd) {
                int rc = flush_frame(S, fr, (uint32_t)fd, gen, host_fd, oflags);
                if (rc < 0 && !err) err = rc;
            }
        }
    }
    return err;
}

/* gunlink: remove the host file; a cached closed copy is invalidated. */
__device__ __noinline__ int st_unlink(gfs_state* S, const char* name) {
    Name nm;
    name_load(name, nm);
    if (nm.len == 0 || nm.len >= GFS_NAME_MAX) return -GFS_EINVAL;
    int slot = file_find(S, nm);
    Waiter w(S->timeout_ns);
    if (slot < 0) {
        if (!spin_lock(&S->table_lock, w)) return -GFS_ETIMEDOUT;
        slot = file_find(S, nm);
        if (slot < 0) slot = file_claim(S, nm);
        spin_unlock(&S->table_lock);
        if (slot < 0) return -GFS_EMFILE;
    }
    gfs_file* fe = &S->files[slot];
    Req r = {};
    r.op = GFS_OP_UNLINK;
    r.file = (uint32_t)slot;
    r.name = fe->name;
    int rc = rpc_call(S, r, file_done(S, (uint32_t)slot));
    uint32_t st = ld_acq(&fe->st);
    if (sstatus(st) == GFS_SS_CLOSED) {
        atomicAdd(&fe->gen, 1u);
        st_rlx64(&fe->cached_ctime, 0ULL);
        st_rlx64(&fe->cached_size, ~0ULL);
    }
    return rc < 0 ? rc : 0;
}

} // namespace
} // namespace gfsd
#endif

/*
 * The reference's kernel-callable file API, same names and signatures as
 * libgpufs/fs_calls.cu.h:34-65, implemented over the GB300 buffer cache.
 *
 * Semantics kept from the reference:
 *   - calls are collective: every thread of the block calls with the same
 *     arguments (warp for the _warp forms); single_thread_* are per-thread;
 *   - gread/gwrite move bytes through HBM page frames; write-once files
 *     (O_GWRONCE) are never read from the host and are OR-merged into the
 *     host file at write-back (host_loop.h:76-137);
 *   - data reaches the host file at gclose (last close), gfsync, gmsync, or
 *     when the clock evictor needs the frame.
 * Differences (a strict superset): errors come back as negative values or
 * GMAP_FAILED instead of compiled-out asserts; gread clamps at end of file
 * and returns the bytes read; gftruncate accepts any size; gunlink works.
 */
#include <stdio.h>
#include "gfs_block.cuh"

/* The file-system state of the current session; set by gfs_create(). */
__device__ gfs_state* g_gfs;

using namespace gfsd;

/* fs_calls.cu:227-236 */
__device__ int gopen(const char* filename, int flags) { return blk_open(g_gfs, filename, flags); }

/* fs_calls.cu:152-225 */
__device__ int single_thread_open(const char* filename, int flags) { return file_open(g_gfs, filename, flags); }

/* fs_calls.cu:35-105 */
__device__ int gclose(int fd) { return blk_close(g_gfs, fd); }

/* fs_calls.cu:689-737 */
__device__ size_t gread(int fd, size_t offset, size_t size, unsigned char* buffer) {
    long long r = blk_read(g_gfs, fd, offset, size, buffer);
    return r < 0 ? (size_t)r : (size_t)r;
}

/* fs_calls.cu:739-802 */
__device__ size_t gwrite(int fd, size_t offset, size_t size, unsigned char* buffer) {
    long long r = blk_write(g_gfs, fd, offset, size, buffer);
    return (size_t)r;
}

/* fs_calls.cu:422-481 */
__device__ volatile void* gmmap(void* addr, size_t size, int prot, int flags, int fd, off_t offset) {
    (void)addr;
    (void)prot;
    (void)flags;
    return (volatile void*)blk_mmap(g_gfs, fd, (uint64_t)offset, size);
}

/* fs_calls.cu:385-401 */
__device__ int gmunmap(volatile void* addr, size_t length) {
    (void)length;
    return blk_munmap(g_gfs, addr);
}

/* fs_calls.cu:618-683: warp-collective mapping; `ref` pins are taken */
__device__ volatile void* gmmap_warp(void* addr, size_t size, int prot, int flags, int fd, off_t offset, int ref) {
    (void)addr;
    (void)prot;
    (void)flags;
    gfs_state* S = g_gfs;
    const unsigned mask = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    int r = 0;
    bool fresh = false;
    MapFill mf = {};
    if (lane == leader) r = map_pin(S, fd, (uint64_t)offset, size, &fresh, ref < 1 ? 1 : ref, &mf);
    r = __shfl_sync(mask, r, leader);
    int fz = __shfl_sync(mask, (int)fresh, leader);
    if (r < 0) return (volatile void*)-1;
    if (fz) {
        /* a missed page of a mapped file is copied from the mapping by the
         * warp (no host request); any other fresh page is zeroed */
        const uint64_t len = __shfl_sync(mask, mf.len, leader);
        const uint64_t src = __shfl_sync(mask, mf.map + ((uint64_t)mf.blk << S->log_page), leader);
        int rank = __popc(mask & ((1u << lane) - 1u)), cnt = __popc(mask);
        uint8_t* d = frame_data(S, (uint32_t)r);
        const uint32_t n16 = (uint32_t)(len >> 4);
        for (uint32_t k = (uint32_t)rank; k < n16; k += (uint32_t)cnt)
            ((uint4*)d)[k] = ((const uint4*)(uintptr_t)src)[k];
        const uint32_t l16 = ((uint32_t)len + 15u) & ~15u;
        for (uint32_t k = n16 * 16u + (uint32_t)rank; k < l16; k += (uint32_t)cnt)
            d[k] = k < (uint32_t)len ? ((const uint8_t*)(uintptr_t)src)[k] : (uint8_t)0;
        for (uint32_t k = l16 + (uint32_t)rank * 16u; k < S->page_size; k += (uint32_t)cnt * 16u)
            *(uint4*)(d + k) = make_uint4(0, 0, 0, 0);
        __syncwarp(mask);
        if (lane == leader) {
            if (len) st_rlx(&S->frames[r].content, (uint32_t)len);
            publish_valid(S, (uint32_t)r);
        }
        __syncwarp(mask);
    }
    return (volatile void*)(frame_data(S, (uint32_t)r) + ((uint64_t)offset & (S->page_size - 1u)));
}

/* fs_calls.cu:403-420 */
__device__ int gmunmap_warp(volatile void* addr, size_t length, int ref) {
    (void)length;
    __threadfence();
    const unsigned mask = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    int r = 0;
    if (lane == leader) r = unmap_one(g_gfs, addr, ref < 1 ? 1 : ref);
    return __shfl_sync(mask, r, leader);
}

/* fs_calls.cu:804-843: write the mapped page back now (single thread) */
__device__ int gmsync(volatile void* addr, size_t length, int flags) {
    (void)length;
    (void)flags;
    gfs_state* S = g_gfs;
    int fr = addr_frame(S, addr);
    if (fr < 0) return -1;
    __threadfence();
    uint64_t key = ld_rlx64(&S->frames[fr].key);
    uint32_t f = key_file(key);
    if (f >= S->n_files) return -1;
    gfs_file* fe = &S->files[f];
    mark_dirty(S, (uint32_t)fr);
    return flush_frame(S, (uint32_t)fr, f, ld_rlx(&fe->gen), (int)ld_rlx((const uint32_t*)&fe->host_fd),
                       (int)ld_rlx((const uint32_t*)&fe->flags));
}

/* fs_calls.cu:107-125 */
__device__ int gfsync(int fd) { return blk_flush(g_gfs, fd); }

__device__ int single_thread_fsync(int fd) { return st_fsync(g_gfs, fd); }

/* fs_calls.cu:127-140 */
__device__ int single_thread_ftruncate(int fd, int size) { return st_truncate(g_gfs, fd, (uint64_t)(size < 0 ? 0 : size)); }

/* fs_calls.cu:143-149 */
__device__ int gftruncate(int fd, int size) {
    __shared__ int s_r;
    __syncthreads();
    if (blk_tid() == 0) s_r = single_thread_ftruncate(fd, size);
    __syncthreads();
    return s_r;
}

/* fs_calls.cu:845-850 (unimplemented in the reference) */
__device__ unsigned int gunlink(char* filename) {
    int r = st_unlink(g_gfs, filename);
    return (unsigned int)(r < 0 ? -r : 0);
}

/* fs_calls.cu:851-854 */
__device__ size_t fstat(int fd) {
    gfs_state* S = g_gfs;
    if (fd < 0 || (uint32_t)fd >= S->n_files) return 0;
    return (size_t)ld_rlx64(&S->files[fd].size);
}

/* device side of the samples' INIT_LOCK / LAST_SEMAPHORE / ERROR helpers */
/* Bytes [off, off + size) of a file opened read-only, addressed straight
 * in its registered host mapping (SM loads over the host link, no cache
 * page); nullptr when the file has no mapping or the range passes its size
 * at open.  Valid while the file stays open. */
__device__ const void* gfs_direct_addr(int fd, unsigned long long off, unsigned long long size) {
    gfs_state* S = g_gfs;
    if (fd < 0 || (uint32_t)fd >= S->n_files) return nullptr;
    gfs_file* fe = &S->files[fd];
    if (sstatus(ld_acq(&fe->st)) != GFS_SS_OPEN) return nullptr;
    if (ld_rlx((const uint32_t*)&fe->flags) != (uint32_t)O_GRDONLY) return nullptr;
    const uint64_t m = ld_rlx64(&fe->map_dev);
    if (!m || off + size > ld_rlx64(&fe->size) || off + size < off) return nullptr;
    return (const void*)(uintptr_t)(m + off);
}

/* ---- fat pointers (include/fat_pointer.cu.h) ----
 * Single-thread page steps the header-only FatPointer template calls; a
 * warp's lanes that want the same page of a file share one call, taking
 * `ref` pins. */

/* pin the page holding byte `off` of fd with `ref` pins; returns the frame
 * or -errno; *fresh: a write-once page the caller must zero and publish */
__device__ int gfs_fp_acquire(int fd, unsigned long long off, int ref, int* fresh) {
    gfs_state* S = g_gfs;
    bool fr = false;
    const unsigned long long page_start = off & ~((unsigned long long)S->page_size - 1ull);
    const int r = map_pin(S, fd, page_start, 0, &fr, ref < 1 ? 1 : ref);
    *fresh = fr ? 1 : 0;
    return r;
}

__device__ unsigned char* gfs_fp_data(int frame) { return frame_data(g_gfs, (uint32_t)frame); }

__device__ void gfs_fp_publish(int frame) { publish_valid(g_gfs, (uint32_t)frame); }

__device__ unsigned int gfs_fp_log_page() { return g_gfs->log_page; }

/* drop `ref` pins of a frame; for a writable file the page is marked dirty
 * and its content and the file's size grow to cover the `touched` bytes of
 * the page (page_start: the page's file offset) */
__device__ void gfs_fp_release(int frame, int ref, unsigned int touched, unsigned long long page_start) {
    gfs_state* S = g_gfs;
    if (frame < 0) return;
    const uint64_t key = ld_rlx64(&S->frames[frame].key);
    const uint32_t f = key_file(key);
    if (f < S->n_files && ld_rlx((const uint32_t*)&S->files[f].flags) != (uint32_t)O_GRDONLY) {
        __threadfence();
        if (touched) {
            atomicMax(&S->frames[frame].content, touched);
            atomicMax((unsigned long long*)&S->files[f].size, page_start + touched);
        }
        mark_dirty(S, (uint32_t)frame);
    }
    unpin(S, (uint32_t)frame, (uint32_t)(ref < 1 ? 1 : ref));
}

/* where a failed translation's accesses go (16 bytes per lane; the
 * session's error bits record the failure) */
__device__ uint4 g_fp_sink[32 * 8];

__device__ unsigned char* gfs_fp_sink() { return (unsigned char*)&g_fp_sink[(threadIdx.x & 31u) * 8u]; }

__device__ unsigned int g_gfs_user_error;
__device__ void gfs_report_user_error(const char* msg, const char* file, int line) {
    atomicOr(&g_gfs_user_error, 1u);
    if (g_gfs) atomicOr(&g_gfs->error, GFS_ERRB_ARG);
    printf("gpufs: %s (%s:%d)\n", msg, file, line);
}
__device__ unsigned long long gfs_globaltimer() { return gtimer(); }

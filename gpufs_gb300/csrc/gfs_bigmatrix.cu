/*
 * bigmatrix_mmap over the GPU file system (samples/bigmatrix_mmap/bigmatrix_mmap.cu:66-168):
 * y = A x with A (rows x cols FP32, row-major) and x read through gmmap, y
 * written through gmmap of a write-once file.
 *
 * Blocks take groups of eight rows from a counter of the launch (the
 * reference gives each block a fixed run of rows) and map the matrix page
 * under the group (the reference's get_row, :45-60, remaps only when the
 * cursor leaves the page).  Where every group lies in one page, the block's
 * last warp pins the next group's page while the others stream the current
 * one, so a block holds at most two matrix pages; otherwise one page is
 * mapped at a time.  Eight whole rows of a page are one pass in which every
 * streaming thread keeps sixteen 16-byte loads in flight; rows are reduced
 * in a fixed order (warp shuffles, then one warp over the partials), so
 * results are deterministic -- the reference adds the per-thread partials
 * with a shared-memory float atomicAdd (:35), whose order varies run to run.
 *
 * This translation unit is compiled without the 64-register cap of the
 * device-API units: the kernel is bounded at 512 threads a block, which
 * leaves each thread the registers of its sixteen loads.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include "fs_calls.cu.h"
#include "gfs_device.cuh"
#include "gfs_block.cuh"
#include "gfs_runtime.h"

extern __device__ gfs_state* g_gfs;

/* gfs_calls.cu: a read-only file's bytes in its registered host mapping */
__device__ const void* gfs_direct_addr(int fd, unsigned long long off, unsigned long long size);
/* gfs_apps.cu */
long long gfs__sum_results(long long* d, int n, cudaStream_t s);

namespace {



/* a group of eight rows taken ahead, with its matrix page pinned */
struct PageAhead {
    unsigned long long g; /* group index (>= the group count: none left) */
    int frame;            /* pinned frame, -1 if none */
    int err;              /* map_pin's error */
    int fresh;            /* the frame still has to be filled (fill) */
    gfsd::MapFill fill;
};

/* block-wide sum of one float per thread, fixed order */
__device__ float block_sum(float v, float* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    float r = 0.f;
    if (warp == 0) {
        r = lane < nw ? red[lane] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xFFFFFFFFu, r, o);
    }
    __syncthreads();
    return r; /* valid in warp 0 */
}

/* partial dot of n floats (a, b 16-byte aligned when n4 path) */
__device__ float dot_part(const float* a, const float* b, uint32_t n) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    const uint32_t n4 = ((((uintptr_t)a | (uintptr_t)b) & 15u) == 0u) ? n / 4u : 0u;
    const float4* a4 = (const float4*)a;
    const float4* b4 = (const float4*)b;
    const uint32_t bd = blockDim.x;
    uint32_t i = threadIdx.x;
    /* two independent 16-byte row loads in flight per thread */
    for (; i + bd < n4; i += 2u * bd) {
        const float4 p0 = __ldcg(a4 + i), p1 = __ldcg(a4 + i + bd);
        const float4 q0 = __ldg(b4 + i), q1 = __ldg(b4 + i + bd);
        s0 = fmaf(p0.x, q0.x, s0); s1 = fmaf(p0.y, q0.y, s1); s2 = fmaf(p0.z, q0.z, s2); s3 = fmaf(p0.w, q0.w, s3);
        s0 = fmaf(p1.x, q1.x, s0); s1 = fmaf(p1.y, q1.y, s1); s2 = fmaf(p1.z, q1.z, s2); s3 = fmaf(p1.w, q1.w, s3);
    }
    for (; i < n4; i += bd) {
        const float4 p = __ldcg(a4 + i), q = __ldg(b4 + i);
        s0 = fmaf(p.x, q.x, s0);
        s1 = fmaf(p.y, q.y, s1);
        s2 = fmaf(p.z, q.z, s2);
        s3 = fmaf(p.w, q.w, s3);
    }
    for (uint32_t i = 4u * n4 + threadIdx.x; i < n; i += blockDim.x) s0 = fmaf(a[i], b[i], s0);
    return (s0 + s1) + (s2 + s3);
}

/* Eight rows at once: a (16-byte aligned) holds rows of stride4 float4s,
 * b the vector.  The first nct threads of the block stream the rows (the
 * others, if any, only join the reduction); each takes two column steps per
 * iteration: two float4s of b and the eight rows' float4s beside each
 * (sixteen 16-byte loads in flight, about 90 registers, which the 512-thread
 * launch bound leaves room for); the eight sums are reduced together in a
 * fixed order.  y[0..7] (shared) are valid after return. */
__device__ __noinline__ void dot_rows8(const float* a, size_t stride4, const float* b, uint32_t n4, float* red, float* y,
                                       uint32_t nct) {
    float s[8];
#pragma unroll
    for (int k = 0; k < 8; k++) s[k] = 0.f;
    const float4* a4 = (const float4*)a;
    const float4* b4 = (const float4*)b;
    const uint32_t bd = nct;
    uint32_t i = threadIdx.x < nct ? threadIdx.x : n4;
    for (; i + bd < n4; i += 2u * bd) {
        const float4 q0 = __ldg(b4 + i), q1 = __ldg(b4 + i + bd);
        float4 p0[8], p1[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            p0[k] = __ldcs(a4 + (size_t)k * stride4 + i);
            p1[k] = __ldcs(a4 + (size_t)k * stride4 + i + bd);
        }
#pragma unroll
        for (int k = 0; k < 8; k++) {
            s[k] = fmaf(p0[k].w, q0.w, fmaf(p0[k].z, q0.z, fmaf(p0[k].y, q0.y, fmaf(p0[k].x, q0.x, s[k]))));
            s[k] = fmaf(p1[k].w, q1.w, fmaf(p1[k].z, q1.z, fmaf(p1[k].y, q1.y, fmaf(p1[k].x, q1.x, s[k]))));
        }
    }
    for (; i < n4; i += bd) {
        const float4 q = __ldg(b4 + i);
        float4 p[8];
#pragma unroll
        for (int k = 0; k < 8; k++) p[k] = __ldcs(a4 + (size_t)k * stride4 + i);
#pragma unroll
        for (int k = 0; k < 8; k++) s[k] = fmaf(p[k].w, q.w, fmaf(p[k].z, q.z, fmaf(p[k].y, q.y, fmaf(p[k].x, q.x, s[k]))));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < 8; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_xor_sync(0xFFFFFFFFu, s[k], o);
    }
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < 8; k++) red[k * 32 + warp] = s[k];
    __syncthreads();
    if (warp == 0)
#pragma unroll
        for (int k = 0; k < 8; k++) {
            float r = lane < nw ? red[k * 32 + lane] : 0.f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xFFFFFFFFu, r, o);
            if (lane == 0) y[k] = r;
        }
    __syncthreads();
}

/* y = A x.  vec/mat/out: device file names; x_buf: cols floats of scratch
 * per block when x does not fit in one page. */
/* direct: read the matrix straight from its registered host mapping when it
 * has one (one pass over a cold matrix: no cache pages, SM loads over the
 * host link) */
__global__ void __launch_bounds__(GFS_BIGMATRIX_THREADS, 1)
    k_bigmatrix(const char* f_v, const char* f_m, const char* f_o, float* x_scratch, long long* res, int direct,
                unsigned int* init_lock, unsigned long long* next_group) {
    __shared__ float red[8 * 32];
    __shared__ float ys[8];
    __shared__ int s_fail;
    __shared__ unsigned long long s_grp[2];
    __shared__ PageAhead s_pa[2];
    const uint32_t page = g_gfs->page_size;
    /* the three opens go out together, from threads of different warps
     * (one host round trip instead of three when the files need one); a
     * block of fewer warps opens them in turn */
    __shared__ int s_fd[3];
    {
        const char* names[3] = {f_m, f_o, f_v};
        const int flags[3] = {O_GRDONLY, O_GWRONCE, O_GRDONLY};
#pragma unroll
        for (int k = 0; k < 3; k++)
            if (threadIdx.x == (32u * (unsigned)k) % blockDim.x) s_fd[k] = single_thread_open(names[k], flags[k]);
        __syncthreads();
    }
    int zfd_m = s_fd[0];
    int zfd_o = s_fd[1];
    int zfd_v = s_fd[2];
    if (zfd_m < 0 || zfd_o < 0 || zfd_v < 0) {
        if (threadIdx.x == 0) res[blockIdx.x] = zfd_m < 0 ? zfd_m : (zfd_o < 0 ? zfd_o : zfd_v);
        if (zfd_m >= 0) gclose(zfd_m);
        if (zfd_o >= 0) gclose(zfd_o);
        if (zfd_v >= 0) gclose(zfd_v);
        return;
    }
    /* the first block truncates the output, the others wait for it
     * (bigmatrix_mmap.cu:88-97, INIT_LOCK) -- but only before their first
     * store of y, so the truncation overlaps their first rows */
    if (threadIdx.x == 0) {
        s_fail = 0;
        if (atomicCAS(init_lock, 0u, 1u) == 0u) {
            single_thread_ftruncate(zfd_o, 0);
            __threadfence();
            atomicExch(init_lock, 2u);
        }
    }
    __syncthreads();
    const uint64_t size_v = fstat(zfd_v) / 4, size_m = fstat(zfd_m) / 4;
    const uint64_t cols = size_v, rows = cols ? size_m / cols : 0;
    long long result = s_fail;
    const float* x = nullptr;
    volatile void* xmap = (volatile void*)-1;
    if (!result && cols) {
        if (cols * 4 <= page) {
            xmap = gmmap(NULL, cols * 4, 0, O_GRDONLY, zfd_v, 0);
            if (xmap == (volatile void*)-1) result = -GFS_EIO;
            x = (const float*)xmap;
        } else {
            float* xs = x_scratch + (size_t)blockIdx.x * cols;
            long long got = (long long)gread(zfd_v, 0, cols * 4, (uchar*)xs);
            if (got != (long long)(cols * 4)) result = got < 0 ? got : -GFS_EIO;
            x = xs;
        }
    }
    volatile uint8_t* mpage = (volatile uint8_t*)-1;
    uint64_t mbase = ~0ull;
    volatile uint8_t* opage = (volatile uint8_t*)-1;
    uint64_t obase = ~0ull;
    /* map the output page holding y[r] (block-collective) and store y there
     * (thread 0; gmunmap of that page later is block-collective, so the
     * store is ordered before it without a barrier of its own) */
    bool inited = false;
    auto put_y = [&](uint64_t r, float y) {
        const uint64_t oo = r * 4, ob = oo / page * page;
        if (!inited) {
            inited = true;
            if (threadIdx.x == 0) {
                const unsigned long long deadline = gfs_globaltimer() + 30000000000ULL;
                while (atomicAdd(init_lock, 0u) != 2u) {
                    if (gfs_globaltimer() > deadline) { s_fail = -GFS_ETIMEDOUT; break; }
                    __nanosleep(1000);
                }
            }
            __syncthreads();
            if (s_fail) { result = s_fail; return; }
        }
        if (ob != obase) {
            if (opage != (volatile uint8_t*)-1) gmunmap(opage, 0);
            uint64_t olen = rows * 4 - ob < page ? rows * 4 - ob : page;
            opage = (volatile uint8_t*)gmmap(NULL, olen, 0, O_GWRONCE, zfd_o, (off_t)ob);
            if (opage == (volatile uint8_t*)-1) { result = -GFS_EIO; obase = ~0ull; return; }
            obase = ob;
        }
        if (threadIdx.x == 0) *(volatile float*)(opage + (oo - ob)) = y;
    };
    /* the matrix page holding byte pb, mapped (block-collective) */
    auto map_m = [&](uint64_t pb) {
        if (pb == mbase) return;
        if (mpage != (volatile uint8_t*)-1) gmunmap(mpage, 0);
        uint64_t mlen = size_m * 4 - pb < page ? size_m * 4 - pb : page;
        mpage = (volatile uint8_t*)gmmap(NULL, mlen, 0, O_GRDONLY, zfd_m, (off_t)pb);
        if (mpage == (volatile uint8_t*)-1) { result = -GFS_EIO; mbase = ~0ull; return; }
        mbase = pb;
    };
    /* one row through the cache; it may span pages: walk its segments */
    auto row_cached = [&](uint64_t r) {
        const uint64_t rbeg = r * cols * 4, rend = rbeg + cols * 4;
        float acc = 0.f;
        for (uint64_t pos = rbeg; pos < rend && !result;) {
            const uint64_t pb = pos / page * page;
            map_m(pb);
            if (result) break;
            const uint64_t seg_end = pb + page < rend ? pb + page : rend;
            acc += dot_part((const float*)(mpage + (pos - pb)), x + (pos - rbeg) / 4, (uint32_t)((seg_end - pos) / 4));
            pos = seg_end;
        }
        if (result) return;
        put_y(r, block_sum(acc, red));
    };
    const bool vec4 = (cols & 3u) == 0u && (((uintptr_t)x) & 15u) == 0u;
    const uint8_t* dm = (direct && !result) ? (const uint8_t*)gfs_direct_addr(zfd_m, 0, size_m * 4) : nullptr;
    /* Rows go in groups of eight, taken from a launch-wide counter: every
     * block stays busy to the end whatever the row count and grid, and no
     * block starts in the middle of a page.  A group inside one mapped page
     * (or anywhere in the direct mapping) is one eight-row pass; any other
     * goes row by row. */
    const uint64_t groups = (rows + 7u) / 8u;
    long long done = 0;
    /* Lookahead form, for a cached matrix whose groups of eight rows each lie
     * inside one page (16-byte aligned rows): the block's last warp takes the
     * next group and pins its page (copying it in from the file's mapping if
     * it missed) while the other warps stream the current one, so no pass
     * waits on a page-index lookup.  The mapper also drops the pin of the
     * group before, whose rows every warp has finished by then. */
    const bool ahead = !dm && vec4 && cols && !result && blockDim.x >= 64u && (blockDim.x & 31u) == 0u &&
                       (uint64_t)page % (8u * cols * 4u) == 0u;
    if (ahead) {
        const uint32_t mw = blockDim.x / 32u - 1u, warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
        auto take = [&](PageAhead* d) {
            d->g = atomicAdd(next_group, 1ull);
            d->err = 0;
            d->fresh = 0;
            d->frame = -1;
            d->fill.len = 0;
            if (d->g >= groups) return;
            const uint64_t pb = d->g * 8u * cols * 4u / page * page;
            bool fr = false;
            const int f = gfsd::map_pin(g_gfs, zfd_m, pb, 0, &fr, 1, &d->fill);
            if (f < 0) {
                d->err = f;
                return;
            }
            d->frame = f;
            d->fresh = fr ? 1 : 0;
        };
        if (threadIdx.x == 0) take(&s_pa[0]);
        __syncthreads();
        /* mapper lane 0: held = the pinned frame of the group in hand, nxt =
         * that of the group taken ahead (both dropped at the end) */
        int held = -1, nxt = s_pa[0].frame;
        for (uint32_t it = 0;; it++) {
            PageAhead& cur = s_pa[it & 1u];
            if (cur.err) {
                result = cur.err;
                break;
            }
            if (cur.g >= groups) break;
            if (cur.fresh) gfsd::blk_fill_fresh(g_gfs, &cur.frame, cur.fill);
            if (warp == mw && lane == 0) {
                if (held >= 0) gfsd::unpin(g_gfs, (uint32_t)held);
                held = cur.frame;
                take(&s_pa[(it + 1u) & 1u]);
                nxt = s_pa[(it + 1u) & 1u].frame;
            }
            const uint64_t r = cur.g * 8u, rn = rows - r < 8u ? rows - r : 8u;
            const uint64_t rbeg = r * cols * 4, pb0 = rbeg / page * page;
            const float* rowp = (const float*)(gfsd::frame_data(g_gfs, (uint32_t)cur.frame) + (rbeg - pb0));
            if (rn == 8u) {
                dot_rows8(rowp, cols / 4, x, (uint32_t)(cols / 4), red, ys, blockDim.x - 32u);
                for (uint64_t k = 0; k < 8u && !result; k++) put_y(r + k, ys[k]);
            } else {
                for (uint64_t k = 0; k < rn && !result; k++) put_y(r + k, block_sum(dot_part(rowp + k * cols, x, (uint32_t)cols), red));
            }
            done += (long long)rn;
            __syncthreads(); /* the next slot is filled; this group's rows are done */
            if (result) break;
        }
        __syncthreads();
        if (warp == mw && lane == 0) {
            if (held >= 0) gfsd::unpin(g_gfs, (uint32_t)held);
            /* a group taken ahead but never started (an error ended the
             * loop after the take; at a normal end there is none).  Its pin
             * is its own even when it shares the frame of the group in hand */
            if (nxt >= 0) gfsd::unpin(g_gfs, (uint32_t)nxt);
        }
    }
    for (uint32_t it = 0; !ahead && !result && cols; it++) {
        if (threadIdx.x == 0) s_grp[it & 1u] = atomicAdd(next_group, 1ull);
        __syncthreads();
        const uint64_t gi = s_grp[it & 1u];
        if (gi >= groups) break;
        const uint64_t r = gi * 8u, rn = rows - r < 8u ? rows - r : 8u;
        const uint64_t rbeg = r * cols * 4, pb0 = rbeg / page * page;
        if (dm && vec4 && rn == 8u) {
            dot_rows8((const float*)(dm + rbeg), cols / 4, x, (uint32_t)(cols / 4), red, ys, blockDim.x);
        } else if (!dm && vec4 && rn == 8u && rbeg + 8 * cols * 4 <= pb0 + page) {
            map_m(pb0);
            if (result) break;
            dot_rows8((const float*)(mpage + (rbeg - pb0)), cols / 4, x, (uint32_t)(cols / 4), red, ys, blockDim.x);
        } else {
            for (uint64_t k = 0; k < rn && !result; k++) {
                if (dm) put_y(r + k, block_sum(dot_part((const float*)(dm + (r + k) * cols * 4), x, (uint32_t)cols), red));
                else row_cached(r + k);
            }
            done += (long long)rn;
            continue;
        }
        for (uint64_t k = 0; k < 8u && !result; k++) put_y(r + k, ys[k]);
        done += 8;
    }
    if (mpage != (volatile uint8_t*)-1) gmunmap(mpage, 0);
    if (opage != (volatile uint8_t*)-1) gmunmap(opage, 0);
    if (xmap != (volatile void*)-1) gmunmap(xmap, 0);
    /* Closes: the block writes back the output first if it is the last to
     * close it (block-collective); then the output's host close and those of
     * the two read-only files (nothing to write back) go out together from
     * threads of different warps, so their host round trips overlap. */
    __shared__ int s_cl[4];
    if (threadIdx.x == 0) s_cl[3] = gfsd::file_close_begin(g_gfs, zfd_o);
    __syncthreads();
    const int yb = s_cl[3];
    const int fl = yb > 0 ? gfsd::blk_flush(g_gfs, zfd_o) : 0;
    {
        const unsigned tm = 32u % blockDim.x, tv = 64u % blockDim.x;
        if (threadIdx.x == 0) s_cl[2] = yb > 0 ? gfsd::file_close_finish(g_gfs, zfd_o) : yb;
        if (threadIdx.x == tm) {
            const int b = gfsd::file_close_begin(g_gfs, zfd_m);
            s_cl[0] = b > 0 ? gfsd::file_close_finish(g_gfs, zfd_m) : b;
        }
        if (threadIdx.x == tv) {
            const int b = gfsd::file_close_begin(g_gfs, zfd_v);
            s_cl[1] = b > 0 ? gfsd::file_close_finish(g_gfs, zfd_v) : b;
        }
    }
    __syncthreads();
    const int c0 = s_cl[0], c1 = s_cl[1], c2 = fl < 0 ? fl : s_cl[2];
    if (threadIdx.x == 0)
        res[blockIdx.x] = result ? result : (c0 < 0 ? c0 : (c1 < 0 ? c1 : (c2 < 0 ? c2 : done)));
}

} // namespace

extern "C" {

void gfs__preload_bigmatrix() {
    cudaFuncAttributes a;
    cudaFuncGetAttributes(&a, k_bigmatrix);
}

static int bigmatrix(gfs_ctx* ctx, const char* vec_path, const char* mat_path, const char* out_path, int nblocks,
                     int nthreads, float* kernel_ms, int direct) {
    if (!vec_path || !mat_path || !out_path || nblocks < 1 || nthreads < 32 || nthreads > GFS_BIGMATRIX_THREADS)
        return -GFS_EINVAL;
    if (strlen(vec_path) >= GFS_NAME_MAX || strlen(mat_path) >= GFS_NAME_MAX || strlen(out_path) >= GFS_NAME_MAX)
        return -GFS_EINVAL;
    if (gfs__activate(ctx)) return -GFS_EIO;
    gfs__premap(ctx, vec_path);
    gfs__premap(ctx, mat_path);
    cudaStream_t s = (cudaStream_t)gfs_kernel_stream(ctx);
    char names[3 * GFS_NAME_MAX];
    memset(names, 0, sizeof names);
    memcpy(names, vec_path, strlen(vec_path));
    memcpy(names + GFS_NAME_MAX, mat_path, strlen(mat_path));
    memcpy(names + 2 * GFS_NAME_MAX, out_path, strlen(out_path));
    char* d = (char*)gfs__scratch(ctx, 256 + sizeof(long long) * (size_t)nblocks);
    if (!d) return -GFS_ENOMEM;
    long long* res = (long long*)(d + 256);
    /* names at 0..191; the launch's control words (the sample's INIT_LOCK
     * and the next row group to take) at 192 and 200, zeroed per launch so
     * that launches of other sessions never share them; results from 256 */
    static_assert(3 * GFS_NAME_MAX <= 192, "names fit before the control words");
    cudaMemcpyAsync(d, names, sizeof names, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(d + 192, 0, 64 + sizeof(long long) * (size_t)nblocks, s);
    unsigned int* init_lock = (unsigned int*)(d + 192);
    unsigned long long* next_group = (unsigned long long*)(d + 200);
    /* x scratch only when x does not fit a page */
    float* xs = nullptr;
    long long vbytes = 0;
    {
        struct stat st;
        if (stat(vec_path, &st) == 0) vbytes = (long long)st.st_size;
    }
    if ((uint64_t)vbytes > gfs_page_size(ctx) && cudaMalloc(&xs, (size_t)vbytes * (size_t)nblocks) != cudaSuccess)
        return -GFS_ENOMEM;
    cudaEvent_t a, b;
    if (kernel_ms) {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, s);
    }
    k_bigmatrix<<<nblocks, nthreads, 0, s>>>(d, d + GFS_NAME_MAX, d + 2 * GFS_NAME_MAX, xs, res, direct, init_lock,
                                             next_group);
    cudaError_t le = cudaGetLastError();
    if (kernel_ms) {
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(kernel_ms, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    long long r = le == cudaSuccess ? gfs__sum_results(res, nblocks, s) : -GFS_EINVAL;
    if (xs) cudaFree(xs);
    return r < 0 ? (int)r : 0;
}

int gfs_bigmatrix(gfs_ctx* ctx, const char* vec_path, const char* mat_path, const char* out_path, int nblocks,
                  int nthreads, float* kernel_ms) {
    return bigmatrix(ctx, vec_path, mat_path, out_path, nblocks, nthreads, kernel_ms, 0);
}

int gfs_bigmatrix_direct(gfs_ctx* ctx, const char* vec_path, const char* mat_path, const char* out_path, int nblocks,
                         int nthreads, float* kernel_ms) {
    return bigmatrix(ctx, vec_path, mat_path, out_path, nblocks, nthreads, kernel_ms, 1);
}

} /* extern "C" */

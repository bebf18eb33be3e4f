/*
 * C-ABI entry points that drive the reference-named device API from the
 * host: each launches one kernel on the session's kernel stream whose
 * blocks call gopen/gread/gwrite/gmmap/... exactly as the reference's
 * samples do, and waits for it.
 *
 *   gfs_pread / gfs_pread_dev   gread path     (libgpufs/fs_calls.cu:689-737)
 *   gfs_pwrite                  gwrite path    (fs_calls.cu:739-802)
 *   gfs_mmap_read               gmmap path     (fs_calls.cu:385-481, 618-683)
 *   gfs_memcopy                 samples/memcopy/cp.cu:73-108 (test_cpy)
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include "fs_calls.cu.h"
#include "gfs_device.cuh"
#include "gfs_runtime.h"

namespace {

struct Names {
    char* a;
    char* b;
    long long* results; /* per-block results */
};

/* copy up to two names and a result array into the session scratch */
int stage(gfs_ctx* c, const char* n1, const char* n2, int nblocks, Names* out) {
    size_t l1 = n1 ? strlen(n1) : 0, l2 = n2 ? strlen(n2) : 0;
    if (l1 >= FILENAME_SIZE || l2 >= FILENAME_SIZE) return -GFS_EINVAL;
    if (nblocks < 1) return -GFS_EINVAL;
    if (gfs__activate(c)) return -GFS_EIO;
    size_t need = 256 + sizeof(long long) * (size_t)nblocks;
    char* s = (char*)gfs__scratch(c, need);
    if (!s) return -GFS_ENOMEM;
    char host[256];
    memset(host, 0, sizeof host);
    if (n1) memcpy(host, n1, l1);
    if (n2) memcpy(host + 128, n2, l2);
    cudaStream_t st = (cudaStream_t)gfs_kernel_stream(c);
    if (cudaMemcpyAsync(s, host, sizeof host, cudaMemcpyHostToDevice, st) != cudaSuccess) return -GFS_EIO;
    if (cudaMemsetAsync(s + 256, 0, sizeof(long long) * (size_t)nblocks, st) != cudaSuccess) return -GFS_EIO;
    out->a = s;
    out->b = s + 128;
    out->results = (long long*)(s + 256);
    return 0;
}

/* Results: smallest negative value if any block failed, else the sum. */
long long collect(gfs_ctx* c, const Names& n, int nblocks) {
    cudaStream_t st = (cudaStream_t)gfs_kernel_stream(c);
    long long* h = new long long[(size_t)nblocks];
    /* wait for the kernel before any copy back: a host copy queued behind a
     * file-system kernel would hold up the workers' own copies it waits on */
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaMemcpy(h, n.results, sizeof(long long) * (size_t)nblocks, cudaMemcpyDeviceToHost);
    long long sum = 0, worst = 0;
    for (int i = 0; i < nblocks && e == cudaSuccess; i++) {
        if (h[i] < 0 && h[i] < worst) worst = h[i];
        if (h[i] > 0) sum += h[i];
    }
    delete[] h;
    if (e != cudaSuccess) {
        fprintf(stderr, "gpufs_gb300: kernel failed: %s\n", cudaGetErrorString(e));
        return -GFS_EIO;
    }
    return worst < 0 ? worst : sum;
}

/* page-aligned slice [*lo, *hi) of [off, off+size) for block b of nb */
__device__ void slice(uint64_t off, uint64_t size, uint32_t page, int b, int nb, uint64_t* lo, uint64_t* hi) {
    uint64_t per = (size + (uint64_t)nb - 1) / (uint64_t)nb;
    per = (per + page - 1) / page * page;
    uint64_t a = off + (uint64_t)b * per;
    uint64_t e = a + per;
    if (a > off + size) a = off + size;
    if (e > off + size) e = off + size;
    *lo = a;
    *hi = e;
}

__global__ void k_pread(const char* name, uint64_t off, uint64_t size, uint8_t* dst, long long* res) {
    int fd = gopen(name, O_GRDONLY);
    if (fd < 0) {
        if (TID == 0) res[blockIdx.x] = fd;
        return;
    }
    uint64_t lo, hi;
    slice(off, size, g_gfs->page_size, blockIdx.x, gridDim.x, &lo, &hi);
    long long got = 0;
    if (hi > lo) got = (long long)gread(fd, lo, hi - lo, dst + (lo - off));
    int c = gclose(fd);
    if (TID == 0) res[blockIdx.x] = got < 0 ? got : (c < 0 ? c : got);
}

__global__ void k_pwrite(const char* name, int oflags, uint64_t off, uint64_t size, const uint8_t* src,
                         long long* res, int do_fsync) {
    int fd = gopen(name, oflags);
    if (fd < 0) {
        if (TID == 0) res[blockIdx.x] = fd;
        return;
    }
    uint64_t lo, hi;
    slice(off, size, g_gfs->page_size, blockIdx.x, gridDim.x, &lo, &hi);
    long long put = 0;
    if (hi > lo) put = (long long)gwrite(fd, lo, hi - lo, (uchar*)(src + (lo - off)));
    if (do_fsync) {
        int s = gfsync(fd);
        if (s < 0 && put >= 0) put = s;
    }
    int c = gclose(fd);
    if (TID == 0) res[blockIdx.x] = put < 0 ? put : (c < 0 ? c : put);
}

__global__ void k_mmap_read(const char* name, uint64_t off, uint64_t size, uint8_t* dst, long long* res, int warp_api) {
    int fd = gopen(name, O_GRDONLY);
    if (fd < 0) {
        if (TID == 0) res[blockIdx.x] = fd;
        return;
    }
    const uint32_t page = g_gfs->page_size;
    uint64_t fsz = fstat(fd);
    uint64_t end = off + size < fsz ? off + size : fsz;
    uint64_t lo, hi;
    slice(off, end > off ? end - off : 0, page, blockIdx.x, gridDim.x, &lo, &hi);
    long long got = 0;
    if (!warp_api) {
        for (uint64_t p = lo; p < hi;) {
            uint64_t pe = (p / page + 1) * page;
            if (pe > hi) pe = hi;
            volatile uchar* m = (volatile uchar*)gmmap(NULL, pe - p, 0, O_GRDONLY, fd, (off_t)p);
            if (m == (volatile uchar*)GMAP_FAILED) { got = -GFS_EIO; break; }
            for (uint64_t k = TID; k < pe - p; k += blockDim.x) dst[p - off + k] = m[k];
            __syncthreads();
            gmunmap(m, 0);
            got += (long long)(pe - p);
            p = pe;
        }
    } else {
        /* each warp maps its own pages */
        const int warp = TID >> 5, nw = (blockDim.x + 31) >> 5, lane = TID & 31;
        uint64_t first = lo / page;
        long long mine = 0;
        for (uint64_t pg = first + (uint64_t)warp; pg * page < hi; pg += (uint64_t)nw) {
            uint64_t p = pg * page > lo ? pg * page : lo;
            uint64_t pe = (pg + 1) * page < hi ? (pg + 1) * page : hi;
            volatile uchar* m = (volatile uchar*)gmmap_warp(NULL, pe - p, 0, O_GRDONLY, fd, (off_t)p, 1);
            if (m == (volatile uchar*)GMAP_FAILED) { mine = -GFS_EIO; break; }
            for (uint64_t k = (uint64_t)lane; k < pe - p; k += 32) dst[p - off + k] = m[k];
            __syncwarp();
            gmunmap_warp(m, 0, 1);
            mine += (long long)(pe - p);
        }
        if (lane == 0) atomicAdd((unsigned long long*)&res[blockIdx.x], (unsigned long long)(mine < 0 ? 0 : mine));
        if (lane == 0 && mine < 0) res[blockIdx.x] = mine;
        __syncthreads();
        got = res[blockIdx.x];
    }
    int c = gclose(fd);
    __syncthreads();
    if (TID == 0) res[blockIdx.x] = got < 0 ? got : (c < 0 ? c : got);
}

__global__ void k_fstat(const char* name, long long* res) {
    int fd = gopen(name, O_GRDONLY);
    if (fd < 0) {
        if (TID == 0) res[0] = fd;
        return;
    }
    long long s = (long long)fstat(fd);
    int c = gclose(fd);
    if (TID == 0) res[0] = c < 0 ? c : s;
}

__global__ void k_truncate(const char* name, int size, long long* res) {
    int fd = gopen(name, O_GRDWR);
    if (fd < 0) {
        if (TID == 0) res[0] = fd;
        return;
    }
    int t = gftruncate(fd, size);
    int c = gclose(fd);
    if (TID == 0) res[0] = t < 0 ? t : c;
}

__global__ void k_unlink(char* name, long long* res) {
    if (TID == 0) res[0] = -(long long)gunlink(name);
}

/* samples/memcopy/cp.cu:73-108 with the page-sized user buffer in global
 * memory (the reference takes it from the device heap). */
__global__ void k_memcopy(const char* src, const char* dst, uint8_t* scratch, int mode, long long* res) {
    __shared__ int zfd, zfd1;
    __shared__ uint64_t filesize;
    int a = gopen(src, O_GRDONLY);
    int b = gopen(dst, O_GWRONCE);
    if (TID == 0) {
        zfd = a;
        zfd1 = b;
        filesize = a >= 0 ? fstat(a) : 0;
    }
    __syncthreads();
    if (zfd < 0 || zfd1 < 0) {
        if (TID == 0) res[blockIdx.x] = zfd < 0 ? zfd : zfd1;
        if (zfd >= 0) gclose(zfd);
        if (zfd1 >= 0) gclose(zfd1);
        return;
    }
    const uint64_t page = g_gfs->page_size;
    long long moved = 0;
    uint8_t* buf = scratch + (size_t)blockIdx.x * page;
    for (uint64_t me = (uint64_t)blockIdx.x * page; me < filesize; me += page * gridDim.x) {
        uint64_t toRead = filesize - me < page ? filesize - me : page;
        if (mode == 0) {
            long long r = (long long)gread(zfd, me, toRead, buf);
            if (r != (long long)toRead) { moved = r < 0 ? r : -GFS_EIO; break; }
            long long w = (long long)gwrite(zfd1, me, toRead, buf);
            if (w != (long long)toRead) { moved = w < 0 ? w : -GFS_EIO; break; }
        } else {
            volatile uchar* s = (volatile uchar*)gmmap(NULL, toRead, 0, O_GRDONLY, zfd, (off_t)me);
            volatile uchar* d = (volatile uchar*)gmmap(NULL, toRead, 0, O_GWRONCE, zfd1, (off_t)me);
            if (s == (volatile uchar*)GMAP_FAILED || d == (volatile uchar*)GMAP_FAILED) { moved = -GFS_EIO; break; }
            const int warp = TID >> 5, lane = TID & 31, nw = (blockDim.x + 31) >> 5;
            uint64_t part = ((toRead + nw - 1) / nw + 15) & ~15ull;
            uint64_t lo = (uint64_t)warp * part;
            if (lo < toRead) {
                uint64_t hi = lo + part < toRead ? lo + part : toRead;
                gfsd::warp_copy((uint8_t*)d + lo, (const uint8_t*)s + lo, hi - lo, lane);
            }
            __syncthreads();
            gmunmap(s, 0);
            gmunmap(d, 0);
        }
        moved += (long long)toRead;
    }
    int c0 = gclose(zfd);
    int c1 = gclose(zfd1);
    if (TID == 0) res[blockIdx.x] = moved < 0 ? moved : (c0 < 0 ? c0 : (c1 < 0 ? c1 : moved));
}

struct Timer {
    cudaEvent_t a = nullptr, b = nullptr;
    cudaStream_t s;
    explicit Timer(cudaStream_t st, bool on) : s(st) {
        if (on) {
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            cudaEventRecord(a, s);
        }
    }
    void stop(float* ms) {
        if (!a) return;
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(ms, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
};

} // namespace

extern "C" {

void gfs__preload_workloads() {
    cudaFuncAttributes a;
    cudaFuncGetAttributes(&a, k_pread);
    cudaFuncGetAttributes(&a, k_pwrite);
    cudaFuncGetAttributes(&a, k_mmap_read);
    cudaFuncGetAttributes(&a, k_fstat);
    cudaFuncGetAttributes(&a, k_truncate);
    cudaFuncGetAttributes(&a, k_unlink);
    cudaFuncGetAttributes(&a, k_memcopy);
}

long long gfs_pread_dev(gfs_ctx* c, const char* path, uint64_t off, uint64_t size, void* dev_out, int nblocks,
                        int nthreads, float* kernel_ms) {
    gfs__premap(c, path);
    Names n;
    int rc = stage(c, path, nullptr, nblocks, &n);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)gfs_kernel_stream(c);
    Timer t(st, kernel_ms != nullptr);
    k_pread<<<nblocks, nthreads, 0, st>>>(n.a, off, size, (uint8_t*)dev_out, n.results);
    if (cudaGetLastError() != cudaSuccess) return -GFS_EINVAL;
    t.stop(kernel_ms);
    return collect(c, n, nblocks);
}

/* Host buffers: where the device reads pageable host memory through the
 * host's page tables, the kernel takes the caller's buffer as it is (its
 * copies cross the host link as they go, both directions at once);
 * otherwise a device buffer from the session pool is copied in or out. */
long long gfs_pread(gfs_ctx* c, const char* path, uint64_t off, uint64_t size, void* host_out, int nblocks,
                    int nthreads) {
    if (gfs__pageable_access(c)) return gfs_pread_dev(c, path, off, size, host_out, nblocks, nthreads, nullptr);
    cudaStream_t st = (cudaStream_t)gfs_kernel_stream(c);
    void* d = size ? gfs__dev_alloc(c, size, st) : nullptr;
    if (size && !d) return -GFS_ENOMEM;
    long long r = gfs_pread_dev(c, path, off, size, d, nblocks, nthreads, nullptr);
    if (r > 0 && cudaMemcpy(host_out, d, (size_t)r, cudaMemcpyDeviceToHost) != cudaSuccess) r = -GFS_EIO;
    gfs__dev_free(c, d, st);
    return r;
}

static long long pwrite_impl(gfs_ctx* c, const char* path, int oflags, uint64_t off, uint64_t size,
                             const void* host_in, int nblocks, int nthreads, int do_fsync) {
    Names n;
    int rc = stage(c, path, nullptr, nblocks, &n);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)gfs_kernel_stream(c);
    const bool direct = gfs__pageable_access(c) != 0;
    void* d = direct ? (void*)host_in : (size ? gfs__dev_alloc(c, size, st) : nullptr);
    if (size && !d) return -GFS_ENOMEM;
    if (!direct && size && cudaMemcpyAsync(d, host_in, size, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        gfs__dev_free(c, d, st);
        return -GFS_EIO;
    }
    k_pwrite<<<nblocks, nthreads, 0, st>>>(n.a, oflags, off, size, (const uint8_t*)d, n.results, do_fsync);
    long long r = cudaGetLastError() == cudaSuccess ? collect(c, n, nblocks) : -GFS_EINVAL;
    if (!direct) gfs__dev_free(c, d, st);
    return r;
}

long long gfs_pwrite(gfs_ctx* c, const char* path, int oflags, uint64_t off, uint64_t size, const void* host_in,
                     int nblocks, int nthreads) {
    return pwrite_impl(c, path, oflags, off, size, host_in, nblocks, nthreads, 0);
}

long long gfs_pwrite_fsync(gfs_ctx* c, const char* path, uint64_t off, uint64_t size, const void* host_in) {
    return pwrite_impl(c, path, O_GRDWR, off, size, host_in, 1, 256, 1);
}

long long gfs_mmap_read(gfs_ctx* c, const char* path, uint64_t off, uint64_t size, void* host_out, int nblocks,
                        int nthreads, int use_warp_api) {
    gfs__premap(c, path);
    Names n;
    int rc = stage(c, path, nullptr, nblocks, &n);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)gfs_kernel_stream(c);
    const bool direct = gfs__pageable_access(c) != 0;
    void* d = direct ? host_out : (size ? gfs__dev_alloc(c, size, st) : nullptr);
    if (size && !d) return -GFS_ENOMEM;
    k_mmap_read<<<nblocks, nthreads, 0, st>>>(n.a, off, size, (uint8_t*)d, n.results, use_warp_api);
    long long r = cudaGetLastError() == cudaSuccess ? collect(c, n, nblocks) : -GFS_EINVAL;
    if (!direct) {
        if (r > 0 && cudaMemcpy(host_out, d, (size_t)r, cudaMemcpyDeviceToHost) != cudaSuccess) r = -GFS_EIO;
        gfs__dev_free(c, d, st);
    }
    return r;
}

long long gfs_fstat_path(gfs_ctx* c, const char* path) {
    Names n;
    int rc = stage(c, path, nullptr, 1, &n);
    if (rc) return rc;
    k_fstat<<<1, 32, 0, (cudaStream_t)gfs_kernel_stream(c)>>>(n.a, n.results);
    return cudaGetLastError() == cudaSuccess ? collect(c, n, 1) : -GFS_EINVAL;
}

int gfs_truncate_path(gfs_ctx* c, const char* path, long long size) {
    Names n;
    int rc = stage(c, path, nullptr, 1, &n);
    if (rc) return rc;
    k_truncate<<<1, 32, 0, (cudaStream_t)gfs_kernel_stream(c)>>>(n.a, (int)size, n.results);
    return cudaGetLastError() == cudaSuccess ? (int)collect(c, n, 1) : -GFS_EINVAL;
}

int gfs_unlink_path(gfs_ctx* c, const char* path) {
    Names n;
    int rc = stage(c, path, nullptr, 1, &n);
    if (rc) return rc;
    k_unlink<<<1, 32, 0, (cudaStream_t)gfs_kernel_stream(c)>>>(n.a, n.results);
    return cudaGetLastError() == cudaSuccess ? (int)collect(c, n, 1) : -GFS_EINVAL;
}

int gfs_memcopy(gfs_ctx* c, const char* src, const char* dst, int nblocks, int nthreads, int mode, float* kernel_ms) {
    gfs__premap(c, src);
    Names n;
    int rc = stage(c, src, dst, nblocks, &n);
    if (rc) return rc;
    uint8_t* scratch = nullptr;
    size_t page = gfs_page_size(c);
    if (mode == 0 && cudaMalloc(&scratch, page * (size_t)nblocks) != cudaSuccess) return -GFS_ENOMEM;
    cudaStream_t st = (cudaStream_t)gfs_kernel_stream(c);
    Timer t(st, kernel_ms != nullptr);
    k_memcopy<<<nblocks, nthreads, 0, st>>>(n.a, n.b, scratch, mode, n.results);
    if (cudaGetLastError() != cudaSuccess) {
        cudaFree(scratch);
        return -GFS_EINVAL;
    }
    t.stop(kernel_ms);
    long long r = collect(c, n, nblocks);
    cudaFree(scratch);
    return r < 0 ? (int)r : 0;
}

} /* extern "C" */

/*
 * XXH64 of files read through the buffer cache (the checksum the memcopy,
 * batched and served forms report), with and without per-call allocation.
 * bigmatrix_mmap lives in gfs_bigmatrix.cu.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <mutex>
#include <vector>

#include "fs_calls.cu.h"
#include "gfs_device.cuh"
#include "gfs_block.cuh"
#include "gfs_xxh64.cuh"
#include "gfs_runtime.h"

extern __device__ gfs_state* g_gfs;


namespace {

/* ---------------- XXH64 (gfs_xxh64.cuh, public xxHash specification) ---------------- */
/* One warp per file: pages are pinned one at a time by lane 0; every 512
 * bytes are staged in shared memory by the whole warp (16 B per lane) and
 * lanes 0..3 run the four accumulator lanes of the stripes over them.  The
 * tail (< 32 bytes) and the final avalanche run on lane 0. */
__global__ void k_xxh64(const int* fds, const uint64_t* sizes, int n, unsigned long long* out, int* err) {
    __shared__ __align__(16) uint8_t stage[8][512 + 32];
    gfs_state* S = g_gfs;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int warps = (int)(blockDim.x >> 5);
    uint8_t* st = stage[wib & 7];
    for (int f = (int)(blockIdx.x * warps) + wib; f < n; f += (int)(gridDim.x * warps)) {
        const uint64_t size = sizes[f];
        gfsd::PinFile pf = gfsd::pin_file(S, fds[f]);
        uint64_t v1 = gfsx::acc_init(0), v2 = gfsx::acc_init(1), v3 = gfsx::acc_init(2), v4 = gfsx::acc_init(3);
        const uint64_t body = size >= 32 ? size / 32 * 32 : 0;
        /* stripes are consumed 512 bytes at a time; a page holds whole 512s */
        int fr = -1;
        uint64_t cur_page = ~0ull;
        int bad = 0;
        for (uint64_t pos = 0; pos < body && !bad; pos += 512) {
            uint64_t pg = pos >> S->log_page;
            if (pg != cur_page) {
                if (lane == 0) {
                    if (fr >= 0) gfsd::unpin(S, (uint32_t)fr);
                    bool fresh;
                    fr = gfsd::pin_page(S, pf, (uint32_t)pg, GFS_PIN_READ, &fresh);
                    if (fr >= 0 && fresh) gfsd::publish_valid(S, (uint32_t)fr);
                }
                fr = __shfl_sync(0xFFFFFFFFu, fr, 0);
                if (fr < 0) { bad = fr; break; }
                cur_page = pg;
            }
            const uint64_t chunk = body - pos < 512 ? body - pos : 512;
            const uint8_t* src = S->pool + ((size_t)fr << S->log_page) + (pos & (S->page_size - 1u));
            if ((uint64_t)lane * 16 < chunk) *(uint4*)(st + lane * 16) = gfsd::ld_cg4(src + lane * 16);
            __syncwarp();
            if (lane < 4) {
                uint64_t v = lane == 0 ? v1 : lane == 1 ? v2 : lane == 2 ? v3 : v4;
                v = gfsx::acc_stripes(v, st, (uint32_t)(chunk / 32), lane);
                if (lane == 0) v1 = v; else if (lane == 1) v2 = v; else if (lane == 2) v3 = v; else v4 = v;
            }
            __syncwarp();
        }
        v1 = __shfl_sync(0xFFFFFFFFu, v1, 0);
        v2 = __shfl_sync(0xFFFFFFFFu, v2, 1);
        v3 = __shfl_sync(0xFFFFFFFFu, v3, 2);
        v4 = __shfl_sync(0xFFFFFFFFu, v4, 3);
        if (lane == 0 && !bad) {
            /* tail bytes [body, size) */
            uint8_t tail[32];
            for (uint64_t q = body; q < size && !bad; q++) {
                uint64_t pg = q >> S->log_page;
                if (pg != cur_page) {
                    if (fr >= 0) gfsd::unpin(S, (uint32_t)fr);
                    bool fresh;
                    fr = gfsd::pin_page(S, pf, (uint32_t)pg, GFS_PIN_READ, &fresh);
                    if (fr >= 0 && fresh) gfsd::publish_valid(S, (uint32_t)fr);
                    if (fr < 0) { bad = fr; break; }
                    cur_page = pg;
                }
                tail[q - body] = S->pool[((size_t)fr << S->log_page) + (q & (S->page_size - 1u))];
            }
            if (!bad) out[f] = gfsx::finish(v1, v2, v3, v4, size, tail);
        }
        if (lane == 0 && fr >= 0) gfsd::unpin(S, (uint32_t)fr);
        bad = __shfl_sync(0xFFFFFFFFu, bad, 0);
        if (lane == 0 && bad) atomicCAS(err, 0, bad);
        __syncwarp();
    }
}

__global__ void k_open_many(const char* names, int n, int oflags, int* fds, uint64_t* sizes) {
    int f = blockIdx.x;
    if (f >= n) return;
    int fd = gfsd::blk_open(g_gfs, names + (size_t)f * GFS_NAME_MAX, oflags);
    if (threadIdx.x == 0) {
        fds[f] = fd;
        sizes[f] = fd >= 0 ? gfsd::ld_rlx64(&g_gfs->files[fd].size) : 0;
    }
}

__global__ void k_close_many(const int* fds, int n, int* rcs) {
    int f = blockIdx.x;
    if (f >= n) return;
    int r = fds[f] >= 0 ? gfsd::blk_close(g_gfs, fds[f]) : 0;
    if (threadIdx.x == 0) rcs[f] = r;
}

} // namespace

/* per-block results of a launch: the sum of the positive ones, or the most
 * negative (an error) */
long long gfs__sum_results(long long* d, int n, cudaStream_t s) {
    long long* h = new long long[(size_t)n];
    cudaError_t e = cudaStreamSynchronize(s); /* kernel first, then copy back */
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(long long) * (size_t)n, cudaMemcpyDeviceToHost);
    long long sum = 0, worst = 0;
    for (int i = 0; i < n; i++) {
        if (h[i] < worst) worst = h[i];
        if (h[i] > 0) sum += h[i];
    }
    delete[] h;
    if (e != cudaSuccess) return -GFS_EIO;
    return worst < 0 ? worst : sum;
}

namespace {
} // namespace

extern "C" {

void gfs__preload_apps() {
    cudaFuncAttributes a;
    cudaFuncGetAttributes(&a, k_xxh64);
    cudaFuncGetAttributes(&a, k_open_many);
    cudaFuncGetAttributes(&a, k_close_many);
}

/* XXH64 of each file (read through the buffer cache), seed 0. */
int gfs_xxh64_files(gfs_ctx* ctx, const char* const* paths, int n, unsigned long long* host_out, float* kernel_ms) {
    if (n < 1) return -GFS_EINVAL;
    for (int i = 0; i < n; i++)
        if (!paths[i] || strlen(paths[i]) >= GFS_NAME_MAX) return -GFS_EINVAL;
    if (gfs__activate(ctx)) return -GFS_EIO;
    cudaStream_t s = (cudaStream_t)gfs_kernel_stream(ctx);
    size_t nb = (size_t)n * GFS_NAME_MAX;
    char* names = nullptr;
    int* fds = nullptr;
    uint64_t* sizes = nullptr;
    unsigned long long* out = nullptr;
    int* err = nullptr;
    char* blk = nullptr;
    size_t total = nb + (size_t)n * (4 + 8 + 8 + 4) + 256;
    if (cudaMalloc(&blk, total) != cudaSuccess) return -GFS_ENOMEM;
    names = blk;
    sizes = (uint64_t*)(blk + ((nb + 15) & ~(size_t)15));
    out = (unsigned long long*)(sizes + n);
    fds = (int*)(out + n);
    err = fds + n;
    int* rcs = err + 1;
    char* hn = new char[nb];
    memset(hn, 0, nb);
    for (int i = 0; i < n; i++) memcpy(hn + (size_t)i * GFS_NAME_MAX, paths[i], strlen(paths[i]));
    cudaMemcpyAsync(names, hn, nb, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(err, 0, 4, s);
    k_open_many<<<n, 64, 0, s>>>(names, n, O_GRDONLY, fds, sizes);
    cudaEvent_t a, b;
    if (kernel_ms) {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, s);
    }
    int warps = 8;
    int grid = (n + warps - 1) / warps;
    k_xxh64<<<grid, warps * 32, 0, s>>>(fds, sizes, n, out, err);
    if (kernel_ms) {
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(kernel_ms, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    k_close_many<<<n, 64, 0, s>>>(fds, n, rcs);
    int herr = 0;
    std::vector<int> hfds((size_t)n);
    cudaError_t e = cudaStreamSynchronize(s); /* kernels first, then copies back */
    if (e == cudaSuccess) e = cudaMemcpy(host_out, out, sizeof(unsigned long long) * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(hfds.data(), fds, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    delete[] hn;
    cudaFree(blk);
    if (e != cudaSuccess) return -GFS_EIO;
    for (int i = 0; i < n; i++)
        if (hfds[(size_t)i] < 0) return hfds[(size_t)i];
    return herr;
}

} /* extern "C" */

/* ---- allocation-free XXH64 over files ----
 * The same three kernels as gfs_xxh64_files, with every per-call buffer
 * (names, sizes, hashes, descriptors, close codes, error word) carved from
 * one file-scope device array of fixed size instead of cudaMalloc.  Its
 * device address is looked up once per device with cudaGetSymbolAddress, so
 * the first call on a device does that set-up (and should come before any
 * stream capture); later calls make no allocation of any kind, on the device
 * or on the host.  All callers on a device share the array: overlapping calls
 * on one device race and must be serialised by the caller. */
namespace {

constexpr size_t XN_NAMES = (size_t)GFS_XXH64_NOALLOC_MAX_FILES * GFS_NAME_MAX;
constexpr size_t XN_SIZES = XN_NAMES;
constexpr size_t XN_OUT = XN_SIZES + 8u * GFS_XXH64_NOALLOC_MAX_FILES;
constexpr size_t XN_FDS = XN_OUT + 8u * GFS_XXH64_NOALLOC_MAX_FILES;
constexpr size_t XN_RCS = XN_FDS + 4u * GFS_XXH64_NOALLOC_MAX_FILES;
constexpr size_t XN_ERR = XN_RCS + 4u * GFS_XXH64_NOALLOC_MAX_FILES;
constexpr size_t XN_BYTES = XN_ERR + 256u;
constexpr int XN_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_xxh64_scratch[XN_BYTES];

unsigned char* g_xxh64_scratch_addr[XN_MAX_DEVICES];
std::mutex g_xxh64_scratch_mu;

/* device address of g_xxh64_scratch on device `dev`, which the caller has
 * made current (set-up on first use on a device).  A cached address is
 * checked against the driver's view of that device's memory on every call
 * (no allocation), so after a device reset it is looked up again. */
int xxh64_scratch(int dev, unsigned char** out) {
    if (dev < 0 || dev >= XN_MAX_DEVICES) return -GFS_EIO;
    std::lock_guard<std::mutex> lk(g_xxh64_scratch_mu);
    if (g_xxh64_scratch_addr[dev]) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, g_xxh64_scratch_addr[dev]) != cudaSuccess || a.type != cudaMemoryTypeDevice ||
            a.device != dev) {
            cudaGetLastError();
            g_xxh64_scratch_addr[dev] = nullptr;
        }
    }
    if (!g_xxh64_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_xxh64_scratch);
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "gpufs_gb300: gfs_xxh64_files_noalloc: cudaGetSymbolAddress failed: %s\n",
                    cudaGetErrorString(e));
            return -GFS_EIO;
        }
        g_xxh64_scratch_addr[dev] = (unsigned char*)p;
    }
    *out = g_xxh64_scratch_addr[dev];
    return 0;
}

} /* namespace */

static int xxh64_noalloc_on_device(gfs_ctx* ctx, int dev, const char* const* paths, int n,
                                   unsigned long long* host_out);

extern "C" int gfs_xxh64_files_noalloc(gfs_ctx* ctx, const char* const* paths, int n, unsigned long long* host_out) {
    if (n < 1 || !paths || !host_out) return -GFS_EINVAL;
    if (n > GFS_XXH64_NOALLOC_MAX_FILES) {
        fprintf(stderr, "gpufs_gb300: gfs_xxh64_files_noalloc: %d files exceed the static scratch limit of %d\n", n,
                GFS_XXH64_NOALLOC_MAX_FILES);
        return -GFS_E2BIG;
    }
    for (int i = 0; i < n; i++)
        if (!paths[i] || strlen(paths[i]) >= GFS_NAME_MAX) return -GFS_EINVAL;
    /* the session's device is current for the call (its stream and the
     * scratch address belong to it); the caller's device comes back after */
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) return -GFS_EIO;
    const int dev = gfs__device(ctx);
    if (prev != dev && cudaSetDevice(dev) != cudaSuccess) return -GFS_EIO;
    const int rc = xxh64_noalloc_on_device(ctx, dev, paths, n, host_out);
    if (prev != dev) cudaSetDevice(prev);
    return rc;
}

static int xxh64_noalloc_on_device(gfs_ctx* ctx, int dev, const char* const* paths, int n,
                                   unsigned long long* host_out) {
    if (gfs__activate(ctx)) return -GFS_EIO;
    unsigned char* base = nullptr;
    int rc = xxh64_scratch(dev, &base);
    if (rc) return rc;
    char* names = (char*)base;
    uint64_t* sizes = (uint64_t*)(base + XN_SIZES);
    unsigned long long* out = (unsigned long long*)(base + XN_OUT);
    int* fds = (int*)(base + XN_FDS);
    int* rcs = (int*)(base + XN_RCS);
    int* err = (int*)(base + XN_ERR);
    cudaStream_t s = (cudaStream_t)gfs_kernel_stream(ctx);
    /* names go up in chunks through a stack buffer: a pageable-to-device
     * cudaMemcpyAsync has consumed its source when it returns */
    constexpr int CH = 32;
    char hn[CH * GFS_NAME_MAX];
    cudaError_t e = cudaSuccess;
    for (int i0 = 0; i0 < n && e == cudaSuccess; i0 += CH) {
        const int m = n - i0 < CH ? n - i0 : CH;
        memset(hn, 0, sizeof hn);
        for (int j = 0; j < m; j++) memcpy(hn + (size_t)j * GFS_NAME_MAX, paths[i0 + j], strlen(paths[i0 + j]));
        e = cudaMemcpyAsync(names + (size_t)i0 * GFS_NAME_MAX, hn, (size_t)m * GFS_NAME_MAX, cudaMemcpyHostToDevice,
                            s);
    }
    /* the error word is the only state that must start at zero */
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, 4, s);
    if (e != cudaSuccess) return -GFS_EIO;
    k_open_many<<<n, 64, 0, s>>>(names, n, O_GRDONLY, fds, sizes);
    const int warps = 8;
    k_xxh64<<<(n + warps - 1) / warps, warps * 32, 0, s>>>(fds, sizes, n, out, err);
    k_close_many<<<n, 64, 0, s>>>(fds, n, rcs);
    e = cudaGetLastError();
    cudaError_t es = cudaStreamSynchronize(s); /* kernels first, then copies back */
    if (e == cudaSuccess) e = es;
    int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpy(host_out, out, sizeof(unsigned long long) * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost);
    int hf[256];
    for (int i0 = 0; i0 < n && e == cudaSuccess; i0 += 256) {
        const int m = n - i0 < 256 ? n - i0 : 256;
        e = cudaMemcpy(hf, fds + i0, 4 * (size_t)m, cudaMemcpyDeviceToHost);
        for (int j = 0; j < m && e == cudaSuccess; j++)
            if (hf[j] < 0) return hf[j];
    }
    if (e != cudaSuccess) return -GFS_EIO;
    return herr;
}

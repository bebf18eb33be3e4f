/*
 * Programs written against the reference's device and host API the way its
 * samples use it (initializer, a kernel on streamMgr->kernelStream calling
 * gopen/fstat/gread/gwrite/gmmap/gmsync/gmunmap/gclose, run_gpufs_handler,
 * delete), compiled with relocatable device code against include/ and
 * linked with libgpufs.a.
 *
 *   copy <src> <dst>    page-by-page copy through a per-block buffer in
 *                       shared memory: every block gread()s pages blockIdx.x,
 *                       blockIdx.x + grid, ... of src and gwrite()s them to a
 *                       new write-once file (the pattern of
 *                       samples/memcopy/cp.cu:73-108);
 *   msync <file> <n>    maps page 0 of an O_GRDWR file, writes a pattern into
 *                       its first n bytes and gmsync()s it; the host reads
 *                       the file while the kernel keeps it open (the device
 *                       waits for the host's acknowledgement, bounded by a
 *                       time limit), after which the kernel writes a second
 *                       pattern, unmaps and closes; the host checks that the
 *                       second pattern landed at close
 *                       (libgpufs/fs_calls.cu:804-843).
 *
 * Exit status 0 and "OK" on success.
 */
#define FS_LOGBLOCKSIZE 14 /* 16 KiB pages: the copy buffer is one page of static shared memory */
#define PPOOL_SIZE (64L << 20)
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include "fs_calls.cu.h"
#include "fs_initializer.cu.h"
#include "host_loop.h"

/* ---- copy ---- */
__global__ void k_copy(const char* src, const char* dst, unsigned long long* bad) {
    __shared__ uchar buf[FS_BLOCKSIZE];
    const int fi = gopen(src, O_GRDONLY);
    const int fo = gopen(dst, O_GWRONCE);
    if (fi < 0 || fo < 0) {
        if (threadIdx.x == 0) atomicAdd(bad, 1ull);
        return;
    }
    const size_t size = fstat(fi);
    for (size_t at = (size_t)blockIdx.x * FS_BLOCKSIZE; at < size; at += (size_t)gridDim.x * FS_BLOCKSIZE) {
        const size_t n = size - at < FS_BLOCKSIZE ? size - at : FS_BLOCKSIZE;
        if (gread(fi, at, n, buf) != n && threadIdx.x == 0) atomicAdd(bad, 1ull);
        if (gwrite(fo, at, n, buf) != n && threadIdx.x == 0) atomicAdd(bad, 1ull);
    }
    gclose(fi);
    gclose(fo);
}

/* ---- msync ---- */
__device__ __host__ static inline uint8_t pat(uint32_t i, uint32_t round) {
    return (uint8_t)((i * 2654435761u + round * 97u) >> 24);
}

/* flag[0]: device -> host "first pattern synced"; flag[1]: host -> device
 * "checked"; flag[2]: device result (0 ok, else a failure code) */
__global__ void k_msync(const char* name, uint32_t n, volatile uint32_t* flag) {
    __shared__ volatile uchar* p;
    __shared__ int fd;
    __shared__ uint32_t res;
    if (threadIdx.x == 0) res = 0;
    fd = gopen(name, O_GRDWR);
    if (fd < 0) {
        if (threadIdx.x == 0) flag[2] = 1;
        return;
    }
    p = (volatile uchar*)gmmap(NULL, FS_BLOCKSIZE, 0, O_GRDWR, fd, 0);
    __syncthreads();
    if (p == GMAP_FAILED) {
        if (threadIdx.x == 0) flag[2] = 2;
        gclose(fd);
        return;
    }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) p[i] = pat(i, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (gmsync(p, FS_BLOCKSIZE, 0) != 0) res = 3;
        __threadfence_system();
        flag[0] = 1;
        /* wait for the host's check, at most about 20 s */
        const unsigned long long t0 = gfs_globaltimer();
        while (flag[1] == 0) {
            if (gfs_globaltimer() - t0 > 20000000000ull) {
                res = 4;
                break;
            }
            __nanosleep(1000);
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) p[i] = pat(i, 2);
    __syncthreads();
    const int um = gmunmap(p, 0); /* block-collective, like gmmap */
    if (threadIdx.x == 0 && um != 0 && res == 0) res = 5;
    __syncthreads();
    if (gclose(fd) != 0 && threadIdx.x == 0 && res == 0) res = 6;
    if (threadIdx.x == 0) flag[2] = res;
}

static int check_file(const char* name, uint32_t n, uint32_t round) {
    FILE* f = fopen(name, "rb");
    if (!f) return -1;
    uint8_t* b = (uint8_t*)malloc(n ? n : 1);
    const size_t got = fread(b, 1, n, f);
    fclose(f);
    int bad = got != n;
    for (uint32_t i = 0; i < n && !bad; i++) bad = b[i] != pat(i, round);
    free(b);
    return bad;
}

int main(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s copy <src> <dst> | msync <file> <n>\n", argv[0]);
        return 2;
    }
    volatile GPUGlobals* gg;
    initializer(&gg);
    cudaStream_t s = gg->streamMgr->kernelStream;
    int rc = 1;
    if (!strcmp(argv[1], "copy")) {
        char *dsrc, *ddst;
        unsigned long long* dbad;
        cudaMalloc(&dsrc, FILENAME_SIZE);
        cudaMalloc(&ddst, FILENAME_SIZE);
        cudaMalloc(&dbad, 8);
        cudaMemset(dbad, 0, 8);
        cudaMemcpy(dsrc, argv[2], strlen(argv[2]) + 1, cudaMemcpyHostToDevice);
        cudaMemcpy(ddst, argv[3], strlen(argv[3]) + 1, cudaMemcpyHostToDevice);
        k_copy<<<28, 256, 0, s>>>(dsrc, ddst, dbad);
        run_gpufs_handler(gg, 0);
        unsigned long long bad = 1;
        cudaMemcpy(&bad, dbad, 8, cudaMemcpyDeviceToHost);
        rc = (cudaGetLastError() == cudaSuccess && bad == 0) ? 0 : 1;
        if (rc) fprintf(stderr, "copy: %llu failed calls\n", bad);
        cudaFree(dsrc);
        cudaFree(ddst);
        cudaFree(dbad);
    } else if (!strcmp(argv[1], "msync")) {
        const uint32_t n = (uint32_t)atoi(argv[3]);
        char* dname;
        cudaMalloc(&dname, FILENAME_SIZE);
        cudaMemcpy(dname, argv[2], strlen(argv[2]) + 1, cudaMemcpyHostToDevice);
        uint32_t* hflag;
        cudaHostAlloc((void**)&hflag, 16, cudaHostAllocMapped);
        memset(hflag, 0, 16);
        hflag[2] = 0xFFFFFFFFu;
        uint32_t* dflag;
        cudaHostGetDevicePointer((void**)&dflag, hflag, 0);
        k_msync<<<1, 128, 0, s>>>(dname, n, (volatile uint32_t*)dflag);
        /* wait for the device's gmsync (at most about 30 s), then check the
         * host file while the kernel still holds it open */
        int synced_ok = 0;
        for (int i = 0; i < 30000 && ((volatile uint32_t*)hflag)[0] == 0; i++) usleep(1000);
        if (((volatile uint32_t*)hflag)[0] == 1) synced_ok = check_file(argv[2], n, 1) == 0;
        ((volatile uint32_t*)hflag)[1] = 1;
        run_gpufs_handler(gg, 0);
        const uint32_t dres = ((volatile uint32_t*)hflag)[2];
        const int closed_ok = check_file(argv[2], n, 2) == 0;
        rc = (synced_ok && closed_ok && dres == 0) ? 0 : 1;
        if (rc) fprintf(stderr, "msync: synced %d closed %d device %u\n", synced_ok, closed_ok, dres);
        cudaFree(dname);
        cudaFreeHost(hflag);
    }
    delete gg;
    if (rc == 0) printf("OK\n");
    return rc;
}

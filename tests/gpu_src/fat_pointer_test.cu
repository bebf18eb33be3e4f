/*
 * Fat pointers (gvmmap / FatPointer, include/fat_pointer.cu.h) exercised the
 * way a GPUfs program uses them: a kernel walks a file of n uint32 values
 * through a read-only fat pointer (grid stride, so every warp crosses 64 KiB
 * pages), writes v * 3 + 1 for each value through a write-once fat pointer,
 * reads scattered positions with moveTo, and steps a copied pointer
 * backwards with -= and operator[].  The host checks the sums, the mismatch
 * counters and the output file byte for byte.  Exit status 0 on success.
 *
 * usage: fat_pointer_test <input file> <output file>
 */
#define FS_LOGBLOCKSIZE 16
#define PPOOL_SIZE (64L << 20)
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include "fs_calls.cu.h"
#include "fs_initializer.cu.h"
#include "host_loop.h"

__device__ __host__ static inline uint32_t pattern(uint64_t i) {
    uint64_t z = i * 0x9E3779B97F4A7C15ull + 0x1234567ull;
    z ^= z >> 29;
    return (uint32_t)(z * 0xBF58476D1CE4E5B9ull >> 32);
}

/* sums[0]: sum of all values read; sums[1]: scattered reads that differ from
 * the pattern; sums[2]: backward reads that differ */
__global__ void k_fp(const char* in, const char* out, uint64_t n, unsigned long long* sums) {
    const int fin = gopen(in, O_GRDONLY);
    const int fout = gopen(out, O_GWRONCE);
    if (fin >= 0 && fout >= 0) {
        const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, T = (uint64_t)gridDim.x * blockDim.x;
        unsigned long long s = 0, bad_scatter = 0, bad_back = 0;
        {
            FatPointer<volatile uint32_t, 32> rp = gvmmap<volatile uint32_t, 32>(NULL, n * 4, 0, O_GRDONLY, fin, 0, NULL);
            FatPointer<uint32_t, 32> wp = gvmmap<uint32_t, 32>(NULL, n * 4, 0, O_GWRONCE, fout, 0, NULL);
            rp.moveTo(tid * 4);
            wp.moveTo(tid * 4);
            for (uint64_t i = tid; i < n; i += T) {
                const uint32_t v = *rp;
                s += v;
                *wp = v * 3u + 1u;
                rp += T;
                wp += T;
            }
            /* scattered reads through a copy of the read pointer */
            FatPointer<volatile uint32_t, 32> sp = rp;
            for (int k = 0; k < 8; k++) {
                const uint64_t i = (tid * 7919u + (uint64_t)k * 104729u) % n;
                sp.moveTo(i * 4);
                if (*sp != pattern(i)) bad_scatter++;
            }
            /* backwards from the thread's last element, and operator[] */
            if (tid < n) {
                const uint64_t last = tid + (n - 1 - tid) / T * T;
                FatPointer<volatile uint32_t, 32> bp = rp;
                bp.moveTo(last * 4);
                for (uint64_t i = last;; i -= T) {
                    if (*bp != pattern(i)) bad_back++;
                    if (i < T) break;
                    bp -= T;
                }
                if (tid + 1 < n && bp[1] != pattern(tid + 1)) bad_back++;
            }
        } /* the pointers release their pages here, before gclose */
        atomicAdd(&sums[0], s);
        atomicAdd(&sums[1], bad_scatter);
        atomicAdd(&sums[2], bad_back);
    } else if (threadIdx.x == 0) {
        atomicAdd(&sums[3], 1ull);
    }
    if (fin >= 0) gclose(fin);
    if (fout >= 0) gclose(fout);
}

int main(int argc, char** argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s in out\n", argv[0]);
        return 2;
    }
    struct stat st;
    if (stat(argv[1], &st) != 0) return 2;
    const uint64_t n = (uint64_t)st.st_size / 4;
    volatile GPUGlobals* g;
    initializer(&g);
    char* names;
    unsigned long long* sums;
    cudaMalloc(&names, 128);
    cudaMalloc(&sums, 4 * sizeof(unsigned long long));
    cudaMemset(names, 0, 128);
    cudaMemset(sums, 0, 4 * sizeof(unsigned long long));
    cudaMemcpy(names, argv[1], strlen(argv[1]), cudaMemcpyHostToDevice);
    cudaMemcpy(names + 64, argv[2], strlen(argv[2]), cudaMemcpyHostToDevice);
    k_fp<<<12, 256, 0, g->streamMgr->kernelStream>>>(names, names + 64, n, sums);
    run_gpufs_handler(g, 0);
    unsigned long long h[4];
    cudaMemcpy(h, sums, sizeof h, cudaMemcpyDeviceToHost);
    unsigned int bits = gfs_last_error(g->ctx, 0);
    delete g;
    unsigned long long want = 0;
    for (uint64_t i = 0; i < n; i++) want += pattern(i);
    int ok = h[0] == want && h[1] == 0 && h[2] == 0 && h[3] == 0 && bits == 0;
    FILE* f = fopen(argv[2], "rb");
    uint64_t bad_out = 0, got_n = 0;
    if (f) {
        uint32_t v;
        while (fread(&v, 4, 1, f) == 1) {
            if (v != pattern(got_n) * 3u + 1u) bad_out++;
            got_n++;
        }
        fclose(f);
    }
    ok = ok && got_n == n && bad_out == 0;
    printf("n=%llu sum=%llu want=%llu bad_scatter=%llu bad_back=%llu open_fail=%llu errbits=0x%x out_n=%llu bad_out=%llu %s\n",
           (unsigned long long)n, h[0], want, h[1], h[2], h[3], bits, (unsigned long long)got_n,
           (unsigned long long)bad_out, ok ? "OK" : "FAIL");
    return ok ? 0 : 1;
}

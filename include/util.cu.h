/*
 * Helpers of the reference's util.cu.h that its samples use
 * (libgpufs/util.cu.h:24-51, 403-433).  Differences: GPU_ASSERT never traps
 * (it reports through the session's error word), INIT_LOCK::try_wait is
 * bounded, and ERROR reports and ends the calling thread instead of raising
 * a device assertion.
 */
#ifndef UTIL_CU_H
#define UTIL_CU_H

#include <stdio.h>
#include <stdlib.h>
#include "fs_constants.h"
#include "fs_debug.cu.h"

#define CUDA_SAFE_CALL(x)                                                                          \
    if ((x) != cudaSuccess) {                                                                      \
        fprintf(stderr, "CUDA ERROR %s: %d %s\n", __FILE__, __LINE__, cudaGetErrorString(cudaGetLastError())); \
        exit(-1);                                                                                  \
    }

__device__ void gfs_report_user_error(const char* msg, const char* file, int line);
__device__ unsigned long long gfs_globaltimer();

#define GPU_ASSERT(x)                                                                              \
    if (!(x)) gfs_report_user_error("assertion failed: " #x, __FILE__, __LINE__);

#define BEGIN_SINGLE_THREAD                                                                        \
    __syncthreads();                                                                               \
    if (threadIdx.x + threadIdx.y + threadIdx.z == 0) {
#define END_SINGLE_THREAD                                                                          \
    }                                                                                              \
    __syncthreads();

#define TID (threadIdx.x + threadIdx.y * blockDim.x + threadIdx.z * blockDim.x * blockDim.y)
#define LANE_ID (TID & 0x1f)
#define WARP_ID (TID >> 5)
#define NUM_WARPS ((blockDim.x * blockDim.y * blockDim.z) >> 5)
#define BLOCK_ID (blockIdx.x + gridDim.x * blockIdx.y + gridDim.x * gridDim.y * blockIdx.z)

struct LAST_SEMAPHORE {
    int count;
    __device__ int is_last() volatile {
        int v = atomicAdd((int*)&count, 1) + 1;
        return v == (int)(gridDim.x * gridDim.y) ? 1 : 0;
    }
};

struct INIT_LOCK {
    volatile int lock;
    /* 1: the caller initialises (then calls signal()); 0: someone else did */
    __device__ int try_wait() volatile {
        int res = atomicMax((int*)&lock, 1);
        if (res == 0) return 1;
        unsigned long long deadline = gfs_globaltimer() + 30000000000ULL;
        while (lock != 2) {
            if (gfs_globaltimer() > deadline) {
                gfs_report_user_error("INIT_LOCK wait timed out", __FILE__, __LINE__);
                break;
            }
            __nanosleep(1000);
        }
        return 0;
    }
    __device__ void signal() volatile {
        __threadfence();
        lock = 2;
        __threadfence();
    }
};

#define ERROR(str)                                                                                 \
    {                                                                                              \
        gfs_report_user_error(str, __FILE__, __LINE__);                                            \
        asm volatile("exit;");                                                                     \
    }

#endif
